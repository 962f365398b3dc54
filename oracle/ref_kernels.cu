// The reference's own CUDA kernels as plain extern "C" entry points.
//
// TEST INFRASTRUCTURE ONLY: the oracle's GPU leg (oracle/ref_gpu.py) loads
// the device code built from this file to run the reference's kernel
// arithmetic on the same GPU as the product, with the reference's build flags
// (-O3 --use_fast_math, native/common.mk:77).
//
// Nothing of the reference is copied here. The reference's kernel sources
// (native/<stage>/kernels/*.cu) are #included from where they lie: the
// recipe in oracle/build_ref.py points the include path at the reference
// tree and selects one stage with -DFXC_REF_<STAGE>. Inside the include, the
// reference's `__global__` kernels are compiled as `__device__` functions;
// each wrapper below is a `__global__` with the reference kernel's exact
// parameter list that calls it, so a launch of the wrapper with the
// reference's grid and block runs the reference kernel unchanged (threadIdx,
// blockIdx, blockDim and dynamic shared memory are the wrapper's). The
// extern "C" names give the loader stable symbols.
//
// Output: device code only (nvcc -cubin), one cubin per stage under
// oracle/_ref/. The host half of each stage (launch order, grid shapes,
// cuFFT calls) is restated in oracle/ref_gpu.py with file:line citations.

#include <assert.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <cstddef>
#include <cstdlib>

#include <cuComplex.h>
#include <cuda_runtime.h>
#include <cuda_runtime_api.h>
#include <cufft.h>
#include <device_launch_parameters.h>
#include <math_constants.h>

#if defined(FXC_REF_SAC2SPEC)
// CUDA 13's cufft.h no longer has these three result codes; the reference's
// error-name helper (native/sac2spec/include/cuda.util.cuh:14-56, host code
// only) still names them in its switch. Distinct stand-in values let that
// header compile unchanged.
#define CUFFT_INCOMPLETE_PARAMETER_LIST ((cufftResult)0x7f01)
#define CUFFT_PARSE_ERROR ((cufftResult)0x7f02)
#define CUFFT_LICENSE_ERROR ((cufftResult)0x7f03)
#endif

#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__

#if defined(FXC_REF_SAC2SPEC)
#include "kernels/complex_matrix.cu"
#include "kernels/rdcrtr.cu"
#include "kernels/real_matrix.cu"
#include "kernels/taper.cu"
#elif defined(FXC_REF_XC)
#include "kernels/cuda.kernels.cu"
#elif defined(FXC_REF_PWS)
#include "kernels/cuda.pws.cu"
#elif defined(FXC_REF_TFPWS)
#include "kernels/cuda.stransform.cu"
#else
#error "select one stage: -DFXC_REF_SAC2SPEC, -DFXC_REF_XC, -DFXC_REF_PWS or -DFXC_REF_TFPWS"
#endif

#pragma pop_macro("__global__")

extern "C" {

#if defined(FXC_REF_SAC2SPEC)
// native/sac2spec/kernels/complex_matrix.cu
__global__ void ref_cisnan2D(cuComplex *d, size_t pitch, size_t width, size_t height)
{
    cisnan2DKernel(d, pitch, width, height);
}
__global__ void ref_cdiv2D(cuComplex *d, size_t dpitch, float *div, size_t spitch, size_t width, size_t height)
{
    cdiv2DKernel(d, dpitch, div, spitch, width, height);
}
__global__ void ref_spectralOnebit2D(cuComplex *d, size_t pitch, size_t width, size_t height, float minval)
{
    spectralOnebit2DKernel(d, pitch, width, height, minval);
}
__global__ void ref_amp2D(float *amp, size_t dpitch, cuComplex *d, size_t spitch, size_t width, size_t height)
{
    amp2DKernel(amp, dpitch, d, spitch, width, height);
}
__global__ void ref_filter(cuComplex *spec, const float *resp, size_t pitch, size_t width, size_t height)
{
    filterKernel(spec, resp, pitch, width, height);
}
__global__ void ref_FwdNormalize2D(cuComplex *d, size_t pitch, size_t width, size_t height, float dt)
{
    FwdNormalize2DKernel(d, pitch, width, height, dt);
}
// native/sac2spec/kernels/rdcrtr.cu
__global__ void ref_sumSingleBlock2D(double *sum, int dpitch, const float *d, int spitch, int width, int height)
{
    sumSingleBlock2DKernel(sum, dpitch, d, spitch, width, height);
}
__global__ void ref_isumSingleBlock2D(double *sum, int dpitch, const float *d, int spitch, int width, int height)
{
    isumSingleBlock2DKernel(sum, dpitch, d, spitch, width, height);
}
__global__ void ref_rdc2D(float *d, int pitch, int width, int height, double *sum)
{
    rdc2DKernel(d, pitch, width, height, sum);
}
__global__ void ref_rtr2D(float *d, int pitch, int width, int height, double *sum, double *isum)
{
    rtr2DKernel(d, pitch, width, height, sum, isum);
}
// native/sac2spec/kernels/real_matrix.cu
__global__ void ref_abs2D(float *d, size_t pitch, size_t width, size_t height)
{
    abs2DKernel(d, pitch, width, height);
}
__global__ void ref_clampmin2D(float *d, size_t pitch, size_t width, size_t height, float minval)
{
    clampmin2DKernel(d, pitch, width, height, minval);
}
__global__ void ref_isnan2D(float *d, size_t pitch, size_t width, size_t height)
{
    isnan2DKernel(d, pitch, width, height);
}
__global__ void ref_div2D(float *d, size_t dpitch, float *div, size_t spitch, size_t width, size_t height)
{
    div2DKernel(d, dpitch, div, spitch, width, height);
}
__global__ void ref_sum2D(float *out, size_t dpitch, float *in, size_t spitch, size_t width, size_t height)
{
    sum2DKernel(out, dpitch, in, spitch, width, height);
}
__global__ void ref_expandSharedWeight2D(float *full, size_t full_pitch, const float *shared, size_t shared_pitch,
                                         size_t width, size_t height, int num_ch)
{
    expandSharedWeight2DKernel(full, full_pitch, shared, shared_pitch, width, height, num_ch);
}
__global__ void ref_cutmax2D(float *d, size_t pitch, size_t width, size_t height, float maxval)
{
    cutmax2DKernel(d, pitch, width, height, maxval);
}
__global__ void ref_onebit2D(float *d, size_t pitch, size_t width, size_t height)
{
    onebit2DKernel(d, pitch, width, height);
}
__global__ void ref_InvNormalize2D(float *d, size_t pitch, size_t width, size_t height, float dt)
{
    InvNormalize2DKernel(d, pitch, width, height, dt);
}
__global__ void ref_smoothRowsRolling(float *out, int dpitch, const float *tmp, int spitch, int width, int height,
                                      int winsize)
{
    smoothRowsRollingKernel(out, dpitch, tmp, spitch, width, height, winsize);
}
// native/sac2spec/kernels/taper.cu
__global__ void ref_specTaper2D(cuComplex *d, size_t pitch, size_t width, size_t height, int np, int idx1, int idx2,
                                int idx3, int idx4)
{
    specTaper2DKernel(d, pitch, width, height, np, idx1, idx2, idx3, idx4);
}
__global__ void ref_timetaper2D(float *d, int pitch, int width, int height, int taper_size)
{
    timetaper2DKernel(d, pitch, width, height, taper_size);
}
#endif  // FXC_REF_SAC2SPEC

#if defined(FXC_REF_XC)
// native/xc/kernels/cuda.kernels.cu
__global__ void ref_generateSignVector(int *sgn, size_t width)
{
    generateSignVector(sgn, width);
}
__global__ void ref_accumulateStepXc2D(const cuComplex *__restrict__ spec, const size_t *__restrict__ src,
                                       const size_t *__restrict__ rec, cuComplex *__restrict__ stack, size_t nspec,
                                       float scale, size_t pair_count)
{
    accumulateStepXc2DKernel(spec, src, rec, stack, nspec, scale, pair_count);
}
__global__ void ref_applyPhaseShift(cuComplex *ncf, int *sgn, size_t spitch, size_t width, size_t height)
{
    applyPhaseShiftKernel(ncf, sgn, spitch, width, height);
}
__global__ void ref_InvNormalize2D(float *d, size_t pitch, size_t width, size_t height, float dt)
{
    InvNormalize2DKernel(d, pitch, width, height, dt);
}
#endif  // FXC_REF_XC

#if defined(FXC_REF_PWS)
// native/pws/kernels/cuda.pws.cu
__global__ void ref_hilbertTransform(cufftComplex *spec, size_t n, size_t ntraces)
{
    hilbertTransformKernel(spec, n, ntraces);
}
__global__ void ref_cudaWeightedMeanBatch(cufftComplex *h, const float *w, const size_t *off, const size_t *cnt,
                                          cufftComplex *mean, size_t num_pairs, size_t nfft)
{
    cudaWeightedMeanBatch(h, w, off, cnt, mean, num_pairs, nfft);
}
__global__ void ref_cudaNormalizeComplex(cufftComplex *h, size_t data_num, size_t nfft)
{
    cudaNormalizeComplex(h, data_num, nfft);
}
__global__ void ref_cudaMultiplyBatch(float *linear, cuComplex *weight, float *pws, size_t num_pairs, size_t nfft)
{
    cudaMultiplyBatch(linear, weight, pws, num_pairs, nfft);
}
#endif  // FXC_REF_PWS

#if defined(FXC_REF_TFPWS)
// native/tfpws/kernels/cuda.stransform.cu
__global__ void ref_hilbertTransform(cufftComplex *spec, size_t n, size_t ntraces)
{
    hilbertTransformKernel(spec, n, ntraces);
}
__global__ void ref_gaussianModulateSub(const cufftComplex *__restrict__ in, cufftComplex *__restrict__ out,
                                        size_t ntraces, size_t n, int f_start, int nf, float scale)
{
    gaussianModulateSub(in, out, ntraces, n, f_start, nf, scale);
}
__global__ void ref_calculateWeightSub(const cufftComplex *__restrict__ sub, const float *__restrict__ w,
                                       cuComplex *__restrict__ wm, size_t n, size_t ntraces, int f_start, int nf)
{
    calculateWeightSub(sub, w, wm, n, ntraces, f_start, nf);
}
__global__ void ref_applyWeight(cufftComplex *tf, cuComplex *wm, size_t nfreq, size_t n, float order)
{
    applyWeight(tf, wm, nfreq, n, order);
}
__global__ void ref_blendBandLimitedSpectrum(cufftComplex *out, const cufftComplex *lin, const cufftComplex *chunk,
                                             int f_start, int nf, float df, float fmin, float fmax, float taper)
{
    blendBandLimitedSpectrum(out, lin, chunk, f_start, nf, df, fmin, fmax, taper);
}
__global__ void ref_sumOverTimeAxis(const cufftComplex *in, cufftComplex *out, size_t nfreq, size_t ntime)
{
    sumOverTimeAxisKernel(in, out, nfreq, ntime);
}
__global__ void ref_extractReal(float *out, cufftComplex *in, size_t nfft)
{
    extractReal(out, in, nfft);
}
#endif  // FXC_REF_TFPWS

}  // extern "C"
