// Device-side mixed-radix FFT used by every stage of the library.
//
// The reference delegates every transform to cuFFT (plans at
// native/sac2spec/device_memory.cu:23-31, native/xc/memory/memory.cu:478-483,
// native/pws/worker/gpu.cu:196-227, native/tfpws/core/tfpws_workspace.cu).
// This file replaces them with one in-shared-memory mixed-radix FFT:
//   * the whole transform of one row lives in one CTA's shared memory
//     (18 522 complex points = 148 KB for the 37 044-point real transform of
//     the xc stage), so each row costs exactly one HBM read and one write;
//   * every stage is an in-place Cooley-Tukey pass (decimation in frequency
//     with digit-reversed output, or its transpose, decimation in time with
//     digit-reversed input), one barrier per stage;
//   * radices 2, 4, 8 are hand-written; odd primes up to 31 use the
//     symmetric real-coefficient DFT; composites 6, 9, 10, 12, 14, 15, 21 run
//     as two small DFTs in registers (one pass over shared memory for two
//     factors); twiddles come from a per-length table
//     computed in double precision on the host and rounded once to float.
// Inverse transforms are forward transforms on conjugated data (the
// conjugation is folded into the first load and the last store).
#pragma once

#include "fxc_common.cuh"

namespace fxc {

constexpr int kFftMaxStages = 24;

struct FftPlan {
  int n;                     // complex transform length
  int nstages;
  int radix[kFftMaxStages];  // radix of each stage, in DIF execution order
  const float2* tw;          // tw[k] = exp(-2*pi*i*k/(n*tw_stride)), k < n*tw_stride
  int tw_stride;             // 1 for a plain complex table, 2 when the table is the real length
  const int* perm;           // perm[k] = point holding frequency k after fft_dif (n entries)
  // b / L_s by a multiply-high: lmag[s] = floor(2^32 / L_s) + 1 for the
  // sub-transform length L_s = n / (radix[0] ... radix[s]) of stage s (the
  // same for the DIF and the DIT pass), exact for b, L_s below 2^16; 0 where
  // L_s == 1. Formed on the host: a 64-bit division per thread and stage runs
  // as FP64 instructions on the GPU.
  uint32_t lmag[kFftMaxStages];
};

__host__ __device__ inline uint32_t fft_lmag(int L) {
  return L > 1 ? (uint32_t)(0x100000000ull / (uint32_t)L) + 1u : 0u;
}

// Host side (fft_plan.cu). composites = false keeps to the prime radices
// and 4, 8 (the row kernels of the stacking stages, whose shared dispatch
// would otherwise carry the composite stages).
int fft_make_plan(int n, const float2* tw, int tw_stride, FftPlan* out, bool composites = true);
// The same with the largest composite radix given (0: none).
int fft_make_plan_limited(int n, const float2* tw, int tw_stride, FftPlan* out, int max_composite);
// The default stages in ascending radix order: the smallest first, the
// largest last (for a transform whose first stage loads its inputs and whose
// last stage is formed at a few frequencies only).
int fft_make_plan_ascending(int n, const float2* tw, int tw_stride, FftPlan* out);
// Cached device table perm[k] = fft_digit_pos(k) for the plan's radix order.
int fft_perm_table(const FftPlan& p, const int** out);
// Its inverse, iperm[fft_digit_pos(k)] = k (cached the same way).
int fft_iperm_table(const FftPlan& p, const int** out);
// Plan whose twiddle and digit-reversal tables are supplied by the caller
// (no device allocation).
int fft_make_plan_with(int n, const float2* tw, int tw_stride, const int* perm, FftPlan* out);
// Host values of the twiddle table exp(-2*pi*i*k/len), k in [0,len), and of
// the digit-reversal table of a plan, as the cached device tables hold them.
void fft_twiddle_values(int len, float2* out);
void fft_perm_values(const FftPlan& p, int* out);
// Returns a cached device table of exp(-2*pi*i*k/len), k in [0,len), for the
// current device. The table lives until process exit.
int fft_twiddles(int len, const float2** out);
bool fft_length_supported(int n);

// cos(2*pi*m/R), sin(2*pi*m/R) for m in [0,R), R in {3,5,7,11,13,17,19,23,29,31}
__constant__ float kOddCos[158] = {
    +1.000000000e+00f, -5.000000000e-01f, -5.000000000e-01f, +1.000000000e+00f,
    +3.090169944e-01f, -8.090169944e-01f, -8.090169944e-01f, +3.090169944e-01f,
    +1.000000000e+00f, +6.234898019e-01f, -2.225209340e-01f, -9.009688679e-01f,
    -9.009688679e-01f, -2.225209340e-01f, +6.234898019e-01f, +1.000000000e+00f,
    +8.412535328e-01f, +4.154150130e-01f, -1.423148383e-01f, -6.548607339e-01f,
    -9.594929736e-01f, -9.594929736e-01f, -6.548607339e-01f, -1.423148383e-01f,
    +4.154150130e-01f, +8.412535328e-01f, +1.000000000e+00f, +8.854560257e-01f,
    +5.680647467e-01f, +1.205366803e-01f, -3.546048870e-01f, -7.485107482e-01f,
    -9.709418174e-01f, -9.709418174e-01f, -7.485107482e-01f, -3.546048870e-01f,
    +1.205366803e-01f, +5.680647467e-01f, +8.854560257e-01f, +1.000000000e+00f,
    +9.324722294e-01f, +7.390089172e-01f, +4.457383558e-01f, +9.226835946e-02f,
    -2.736629901e-01f, -6.026346364e-01f, -8.502171357e-01f, -9.829730997e-01f,
    -9.829730997e-01f, -8.502171357e-01f, -6.026346364e-01f, -2.736629901e-01f,
    +9.226835946e-02f, +4.457383558e-01f, +7.390089172e-01f, +9.324722294e-01f,
    +1.000000000e+00f, +9.458172417e-01f, +7.891405094e-01f, +5.469481581e-01f,
    +2.454854871e-01f, -8.257934547e-02f, -4.016954247e-01f, -6.772815716e-01f,
    -8.794737512e-01f, -9.863613034e-01f, -9.863613034e-01f, -8.794737512e-01f,
    -6.772815716e-01f, -4.016954247e-01f, -8.257934547e-02f, +2.454854871e-01f,
    +5.469481581e-01f, +7.891405094e-01f, +9.458172417e-01f, +1.000000000e+00f,
    +9.629172873e-01f, +8.544194045e-01f, +6.825531432e-01f, +4.600650377e-01f,
    +2.034560131e-01f, -6.824241336e-02f, -3.348796122e-01f, -5.766803221e-01f,
    -7.757112907e-01f, -9.172113015e-01f, -9.906859460e-01f, -9.906859460e-01f,
    -9.172113015e-01f, -7.757112907e-01f, -5.766803221e-01f, -3.348796122e-01f,
    -6.824241336e-02f, +2.034560131e-01f, +4.600650377e-01f, +6.825531432e-01f,
    +8.544194045e-01f, +9.629172873e-01f, +1.000000000e+00f, +9.766205557e-01f,
    +9.075754197e-01f, +7.960930657e-01f, +6.473862848e-01f, +4.684084407e-01f,
    +2.675283385e-01f, +5.413890859e-02f, -1.617819966e-01f, -3.701381553e-01f,
    -5.611870654e-01f, -7.259954919e-01f, -8.568571762e-01f, -9.476531712e-01f,
    -9.941379572e-01f, -9.941379572e-01f, -9.476531712e-01f, -8.568571762e-01f,
    -7.259954919e-01f, -5.611870654e-01f, -3.701381553e-01f, -1.617819966e-01f,
    +5.413890859e-02f, +2.675283385e-01f, +4.684084407e-01f, +6.473862848e-01f,
    +7.960930657e-01f, +9.075754197e-01f, +9.766205557e-01f, +1.000000000e+00f,
    +9.795299413e-01f, +9.189578116e-01f, +8.207634412e-01f, +6.889669191e-01f,
    +5.289640103e-01f, +3.473052528e-01f, +1.514277775e-01f, -5.064916884e-02f,
    -2.506525323e-01f, -4.403941516e-01f, -6.121059825e-01f, -7.587581227e-01f,
    -8.743466161e-01f, -9.541392564e-01f, -9.948693234e-01f, -9.948693234e-01f,
    -9.541392564e-01f, -8.743466161e-01f, -7.587581227e-01f, -6.121059825e-01f,
    -4.403941516e-01f, -2.506525323e-01f, -5.064916884e-02f, +1.514277775e-01f,
    +3.473052528e-01f, +5.289640103e-01f, +6.889669191e-01f, +8.207634412e-01f,
    +9.189578116e-01f, +9.795299413e-01f};
__constant__ float kOddSin[158] = {
    +0.000000000e+00f, +8.660254038e-01f, -8.660254038e-01f, +0.000000000e+00f,
    +9.510565163e-01f, +5.877852523e-01f, -5.877852523e-01f, -9.510565163e-01f,
    +0.000000000e+00f, +7.818314825e-01f, +9.749279122e-01f, +4.338837391e-01f,
    -4.338837391e-01f, -9.749279122e-01f, -7.818314825e-01f, +0.000000000e+00f,
    +5.406408175e-01f, +9.096319954e-01f, +9.898214419e-01f, +7.557495744e-01f,
    +2.817325568e-01f, -2.817325568e-01f, -7.557495744e-01f, -9.898214419e-01f,
    -9.096319954e-01f, -5.406408175e-01f, +0.000000000e+00f, +4.647231720e-01f,
    +8.229838659e-01f, +9.927088741e-01f, +9.350162427e-01f, +6.631226582e-01f,
    +2.393156643e-01f, -2.393156643e-01f, -6.631226582e-01f, -9.350162427e-01f,
    -9.927088741e-01f, -8.229838659e-01f, -4.647231720e-01f, +0.000000000e+00f,
    +3.612416662e-01f, +6.736956436e-01f, +8.951632914e-01f, +9.957341763e-01f,
    +9.618256432e-01f, +7.980172273e-01f, +5.264321629e-01f, +1.837495178e-01f,
    -1.837495178e-01f, -5.264321629e-01f, -7.980172273e-01f, -9.618256432e-01f,
    -9.957341763e-01f, -8.951632914e-01f, -6.736956436e-01f, -3.612416662e-01f,
    +0.000000000e+00f, +3.246994692e-01f, +6.142127127e-01f, +8.371664783e-01f,
    +9.694002659e-01f, +9.965844930e-01f, +9.157733267e-01f, +7.357239107e-01f,
    +4.759473930e-01f, +1.645945903e-01f, -1.645945903e-01f, -4.759473930e-01f,
    -7.357239107e-01f, -9.157733267e-01f, -9.965844930e-01f, -9.694002659e-01f,
    -8.371664783e-01f, -6.142127127e-01f, -3.246994692e-01f, +0.000000000e+00f,
    +2.697967712e-01f, +5.195839500e-01f, +7.308359643e-01f, +8.878852184e-01f,
    +9.790840877e-01f, +9.976687692e-01f, +9.422609221e-01f, +8.169698930e-01f,
    +6.310879443e-01f, +3.984010898e-01f, +1.361666491e-01f, -1.361666491e-01f,
    -3.984010898e-01f, -6.310879443e-01f, -8.169698930e-01f, -9.422609221e-01f,
    -9.976687692e-01f, -9.790840877e-01f, -8.878852184e-01f, -7.308359643e-01f,
    -5.195839500e-01f, -2.697967712e-01f, +0.000000000e+00f, +2.149704402e-01f,
    +4.198891016e-01f, +6.051742152e-01f, +7.621620551e-01f, +8.835120444e-01f,
    +9.635499925e-01f, +9.985334139e-01f, +9.868265225e-01f, +9.289767198e-01f,
    +8.276889982e-01f, +6.876994589e-01f, +5.155538572e-01f, +3.193015301e-01f,
    +1.081190184e-01f, -1.081190184e-01f, -3.193015301e-01f, -5.155538572e-01f,
    -6.876994589e-01f, -8.276889982e-01f, -9.289767198e-01f, -9.868265225e-01f,
    -9.985334139e-01f, -9.635499925e-01f, -8.835120444e-01f, -7.621620551e-01f,
    -6.051742152e-01f, -4.198891016e-01f, -2.149704402e-01f, +0.000000000e+00f,
    +2.012985201e-01f, +3.943558551e-01f, +5.712682151e-01f, +7.247927872e-01f,
    +8.486442575e-01f, +9.377521321e-01f, +9.884683243e-01f, +9.987165072e-01f,
    +9.680771189e-01f, +8.978045396e-01f, +7.907757369e-01f, +6.513724827e-01f,
    +4.853019625e-01f, +2.993631230e-01f, +1.011683220e-01f, -1.011683220e-01f,
    -2.993631230e-01f, -4.853019625e-01f, -6.513724827e-01f, -7.907757369e-01f,
    -8.978045396e-01f, -9.680771189e-01f, -9.987165072e-01f, -9.884683243e-01f,
    -9.377521321e-01f, -8.486442575e-01f, -7.247927872e-01f, -5.712682151e-01f,
    -3.943558551e-01f, -2.012985201e-01f};
// offsets: R3:0, R5:3, R7:8, R11:15, R13:26, R17:39, R19:56, R23:75, R29:98, R31:127

// cos(2*pi*m/R), sin(2*pi*m/R) for m in [0,R), composite R in {6,9,10,12,14,15,21}
__constant__ float kCompCos[87] = {
    +1.000000000e+00f, +5.000000000e-01f, -5.000000000e-01f, -1.000000000e+00f,
    -5.000000000e-01f, +5.000000000e-01f, +1.000000000e+00f, +7.660444431e-01f,
    +1.736481777e-01f, -5.000000000e-01f, -9.396926208e-01f, -9.396926208e-01f,
    -5.000000000e-01f, +1.736481777e-01f, +7.660444431e-01f, +1.000000000e+00f,
    +8.090169944e-01f, +3.090169944e-01f, -3.090169944e-01f, -8.090169944e-01f,
    -1.000000000e+00f, -8.090169944e-01f, -3.090169944e-01f, +3.090169944e-01f,
    +8.090169944e-01f, +1.000000000e+00f, +8.660254038e-01f, +5.000000000e-01f,
    +6.123233996e-17f, -5.000000000e-01f, -8.660254038e-01f, -1.000000000e+00f,
    -8.660254038e-01f, -5.000000000e-01f, -1.836970199e-16f, +5.000000000e-01f,
    +8.660254038e-01f, +1.000000000e+00f, +9.009688679e-01f, +6.234898019e-01f,
    +2.225209340e-01f, -2.225209340e-01f, -6.234898019e-01f, -9.009688679e-01f,
    -1.000000000e+00f, -9.009688679e-01f, -6.234898019e-01f, -2.225209340e-01f,
    +2.225209340e-01f, +6.234898019e-01f, +9.009688679e-01f, +1.000000000e+00f,
    +9.135454576e-01f, +6.691306064e-01f, +3.090169944e-01f, -1.045284633e-01f,
    -5.000000000e-01f, -8.090169944e-01f, -9.781476007e-01f, -9.781476007e-01f,
    -8.090169944e-01f, -5.000000000e-01f, -1.045284633e-01f, +3.090169944e-01f,
    +6.691306064e-01f, +9.135454576e-01f,
    +1.000000000e+00f, +9.555728058e-01f, +8.262387743e-01f, +6.234898019e-01f, +3.653410244e-01f, +7.473009359e-02f, -2.225209340e-01f, -5.000000000e-01f, -7.330518718e-01f, -9.009688679e-01f, -9.888308262e-01f, -9.888308262e-01f, -9.009688679e-01f, -7.330518718e-01f, -5.000000000e-01f, -2.225209340e-01f, +7.473009359e-02f, +3.653410244e-01f, +6.234898019e-01f, +8.262387743e-01f, +9.555728058e-01f
};
__constant__ float kCompSin[87] = {
    +0.000000000e+00f, +8.660254038e-01f, +8.660254038e-01f, +1.224646799e-16f,
    -8.660254038e-01f, -8.660254038e-01f, +0.000000000e+00f, +6.427876097e-01f,
    +9.848077530e-01f, +8.660254038e-01f, +3.420201433e-01f, -3.420201433e-01f,
    -8.660254038e-01f, -9.848077530e-01f, -6.427876097e-01f, +0.000000000e+00f,
    +5.877852523e-01f, +9.510565163e-01f, +9.510565163e-01f, +5.877852523e-01f,
    +1.224646799e-16f, -5.877852523e-01f, -9.510565163e-01f, -9.510565163e-01f,
    -5.877852523e-01f, +0.000000000e+00f, +5.000000000e-01f, +8.660254038e-01f,
    +1.000000000e+00f, +8.660254038e-01f, +5.000000000e-01f, +1.224646799e-16f,
    -5.000000000e-01f, -8.660254038e-01f, -1.000000000e+00f, -8.660254038e-01f,
    -5.000000000e-01f, +0.000000000e+00f, +4.338837391e-01f, +7.818314825e-01f,
    +9.749279122e-01f, +9.749279122e-01f, +7.818314825e-01f, +4.338837391e-01f,
    +1.224646799e-16f, -4.338837391e-01f, -7.818314825e-01f, -9.749279122e-01f,
    -9.749279122e-01f, -7.818314825e-01f, -4.338837391e-01f, +0.000000000e+00f,
    +4.067366431e-01f, +7.431448255e-01f, +9.510565163e-01f, +9.945218954e-01f,
    +8.660254038e-01f, +5.877852523e-01f, +2.079116908e-01f, -2.079116908e-01f,
    -5.877852523e-01f, -8.660254038e-01f, -9.945218954e-01f, -9.510565163e-01f,
    -7.431448255e-01f, -4.067366431e-01f,
    +0.000000000e+00f, +2.947551744e-01f, +5.633200581e-01f, +7.818314825e-01f, +9.308737486e-01f, +9.972037972e-01f, +9.749279122e-01f, +8.660254038e-01f, +6.801727378e-01f, +4.338837391e-01f, +1.490422662e-01f, -1.490422662e-01f, -4.338837391e-01f, -6.801727378e-01f, -8.660254038e-01f, -9.749279122e-01f, -9.972037972e-01f, -9.308737486e-01f, -7.818314825e-01f, -5.633200581e-01f, -2.947551744e-01f
};
// offsets: R6:0, R9:6, R10:15, R12:25, R14:37, R15:51, R21:66

template <int R>
struct OddRadixOffset;
template <> struct OddRadixOffset<3> { static constexpr int v = 0; };
template <> struct OddRadixOffset<5> { static constexpr int v = 3; };
template <> struct OddRadixOffset<7> { static constexpr int v = 8; };
template <> struct OddRadixOffset<11> { static constexpr int v = 15; };
template <> struct OddRadixOffset<13> { static constexpr int v = 26; };
template <> struct OddRadixOffset<17> { static constexpr int v = 39; };
template <> struct OddRadixOffset<19> { static constexpr int v = 56; };
template <> struct OddRadixOffset<23> { static constexpr int v = 75; };
template <> struct OddRadixOffset<29> { static constexpr int v = 98; };
template <> struct OddRadixOffset<31> { static constexpr int v = 127; };

// ---- in-register forward DFT kernels -------------------------------------

__device__ __forceinline__ void dft2(float2 (&x)[2]) {
  float2 a = x[0], b = x[1];
  x[0] = cadd(a, b);
  x[1] = csub(a, b);
}

__device__ __forceinline__ void dft4_vals(float2& b0, float2& b1, float2& b2, float2& b3) {
  float2 t0 = cadd(b0, b2), t1 = csub(b0, b2), t2 = cadd(b1, b3), t3 = csub(b1, b3);
  b0 = cadd(t0, t2);
  b2 = csub(t0, t2);
  b1 = cadd(t1, mul_mi(t3));
  b3 = cadd(t1, mul_pi(t3));
}

__device__ __forceinline__ void dft4(float2 (&x)[4]) { dft4_vals(x[0], x[1], x[2], x[3]); }

__device__ __forceinline__ void dft8(float2 (&x)[8]) {
  const float h = 0.70710678118654752f;
  float2 a0 = cadd(x[0], x[4]), a4 = csub(x[0], x[4]);
  float2 a1 = cadd(x[1], x[5]), a5 = csub(x[1], x[5]);
  float2 a2 = cadd(x[2], x[6]), a6 = csub(x[2], x[6]);
  float2 a3 = cadd(x[3], x[7]), a7 = csub(x[3], x[7]);
  // a5 *= exp(-i pi/4), a6 *= -i, a7 *= exp(-3 i pi/4)
  a5 = make_float2(h * (a5.x + a5.y), h * (a5.y - a5.x));
  a6 = mul_mi(a6);
  a7 = make_float2(h * (a7.y - a7.x), -h * (a7.x + a7.y));
  dft4_vals(a0, a1, a2, a3);
  dft4_vals(a4, a5, a6, a7);
  x[0] = a0; x[2] = a1; x[4] = a2; x[6] = a3;
  x[1] = a4; x[3] = a5; x[5] = a6; x[7] = a7;
}

// Odd-length DFT through the symmetric form
//   y_k = x0 + sum_j (x_j + x_{R-j}) cos(2 pi jk/R) - i (x_j - x_{R-j}) sin(2 pi jk/R)
template <int R>
__device__ __forceinline__ void dft_odd(float2 (&x)[R]) {
  constexpr int H = (R - 1) / 2;
  constexpr int OFF = OddRadixOffset<R>::v;
  float2 a[H], b[H];
#pragma unroll
  for (int j = 1; j <= H; ++j) {
    a[j - 1] = cadd(x[j], x[R - j]);
    b[j - 1] = csub(x[j], x[R - j]);
  }
  float2 y0 = x[0];
#pragma unroll
  for (int j = 0; j < H; ++j) y0 = cadd(y0, a[j]);
  float2 y[R];
#pragma unroll
  for (int k = 1; k <= H; ++k) {
    float2 A = x[0];
    float2 B = make_float2(0.f, 0.f);
#pragma unroll
    for (int j = 1; j <= H; ++j) {
      const int m = (j * k) % R;
      const float c = kOddCos[OFF + m];
      const float s = kOddSin[OFF + m];
      A.x = fmaf(a[j - 1].x, c, A.x);
      A.y = fmaf(a[j - 1].y, c, A.y);
      B.x = fmaf(b[j - 1].x, s, B.x);
      B.y = fmaf(b[j - 1].y, s, B.y);
    }
    y[k] = make_float2(A.x + B.y, A.y - B.x);
    y[R - k] = make_float2(A.x - B.y, A.y + B.x);
  }
  x[0] = y0;
#pragma unroll
  for (int k = 1; k < R; ++k) x[k] = y[k];
}

template <int R>
struct CompRadixOffset;
template <> struct CompRadixOffset<6> { static constexpr int v = 0; };
template <> struct CompRadixOffset<9> { static constexpr int v = 6; };
template <> struct CompRadixOffset<10> { static constexpr int v = 15; };
template <> struct CompRadixOffset<12> { static constexpr int v = 25; };
template <> struct CompRadixOffset<14> { static constexpr int v = 37; };
template <> struct CompRadixOffset<15> { static constexpr int v = 51; };
template <> struct CompRadixOffset<21> { static constexpr int v = 66; };

template <int R>
__device__ __forceinline__ void dft_any(float2 (&x)[R]);

// Composite R = R1 * R2 in registers (one shared-memory pass instead of
// two): with n = R2 n1 + n2 and k = k1 + R1 k2,
//   X[k] = sum_n2 W_R^(n2 k1) W_R2^(n2 k2) sum_n1 x[n] W_R1^(n1 k1),
// i.e. R2 DFTs of length R1, the inner twiddles W_R^(n2 k1), then R1 DFTs
// of length R2; natural order in and out.
template <int R1, int R2>
__device__ __forceinline__ void dft_comp(float2 (&x)[R1 * R2]) {
  constexpr int R = R1 * R2;
  constexpr int OFF = CompRadixOffset<R>::v;
  float2 y[R];  // y[n2 * R1 + k1]
#pragma unroll
  for (int n2 = 0; n2 < R2; ++n2) {
    float2 a[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; ++n1) a[n1] = x[R2 * n1 + n2];
    dft_any<R1>(a);
#pragma unroll
    for (int k1 = 0; k1 < R1; ++k1) {
      const int m = (n2 * k1) % R;
      if (m == 0) {
        y[n2 * R1 + k1] = a[k1];
      } else {
        // a * exp(-2 pi i m / R)
        const float c = kCompCos[OFF + m], sn = kCompSin[OFF + m];
        y[n2 * R1 + k1] = make_float2(fmaf(a[k1].x, c, a[k1].y * sn), fmaf(a[k1].y, c, -a[k1].x * sn));
      }
    }
  }
#pragma unroll
  for (int k1 = 0; k1 < R1; ++k1) {
    float2 b[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; ++n2) b[n2] = y[n2 * R1 + k1];
    dft_any<R2>(b);
#pragma unroll
    for (int k2 = 0; k2 < R2; ++k2) x[k1 + R1 * k2] = b[k2];
  }
}

template <int R>
__device__ __forceinline__ void dft_any(float2 (&x)[R]) {
  if constexpr (R == 2) {
    dft2(x);
  } else if constexpr (R == 4) {
    dft4(x);
  } else if constexpr (R == 8) {
    dft8(x);
  } else if constexpr (R == 6) {
    dft_comp<2, 3>(x);
  } else if constexpr (R == 9) {
    dft_comp<3, 3>(x);
  } else if constexpr (R == 10) {
    dft_comp<2, 5>(x);
  } else if constexpr (R == 12) {
    dft_comp<4, 3>(x);
  } else if constexpr (R == 14) {
    dft_comp<2, 7>(x);
  } else if constexpr (R == 15) {
    dft_comp<3, 5>(x);
  } else if constexpr (R == 21) {
    dft_comp<3, 7>(x);
  } else {
    dft_odd<R>(x);
  }
}

// ---- in-place mixed-radix stages -----------------------------------------
// Stage s (radix r = p.radix[s]) works on blocks of B = r * L points, where
// L = n / (r_0 ... r_s). Butterfly (block, j), j < L, owns the points
// block*B + j + t*L (t < r) and writes its results back to the same points,
// so only one butterfly is live per thread and one barrier ends a stage.
//   DIF (natural order in, digit-reversed out):  y_t = w_B^{t j} * DFT_r(x)_t
//   DIT (digit-reversed in, natural order out):  y = DFT_r(w_B^{t j} * x_t)
// The DIT stages are the transposes of the DIF stages run in reverse order,
// so DIT(DIF(x)) with one of them inverse returns n*x. The point that holds
// frequency k after a DIF is fft_digit_pos(k) (table fft_perm).

// Stage twiddles w^k (k < n*tw_stride) come from a two-level table in shared
// memory: w^k = coarse[k >> 8] * fine[k & 255], both entries of the global
// table copied by fft_twiddles_to_smem (about 3 KB for the longest rows).
// The fine table keeps one unused slot after every 16 entries: a stage reads
// fine[(j * step) & 255] across the lanes' j, and for steps of 16 (or 32 x an
// odd factor) the unpadded entries fall 16 (or 8) to a shared-memory bank;
// padded, they land on distinct banks.
constexpr int kTwFineShift = 8;
constexpr int kTwFine = 1 << kTwFineShift;
constexpr int kTwFinePadded = kTwFine + kTwFine / 16;

__host__ __device__ inline int tw_fine_slot(int i) { return i + (i >> 4); }

__host__ __device__ inline int fft_tw_smem_elems(const FftPlan& p) {
  const int nt = p.n * p.tw_stride;
  return kTwFinePadded + (nt - 1) / kTwFine + 1;
}

// All T threads copy; the caller synchronises before the first stage.
template <int T>
__device__ __forceinline__ void fft_twiddles_to_smem(const FftPlan& p, float2* stw) {
  const int nt = p.n * p.tw_stride;
  for (int i = threadIdx.x; i < kTwFine; i += T)
    stw[tw_fine_slot(i)] = i < nt ? __ldg(p.tw + i) : make_float2(1.f, 0.f);
  const int nc = (nt - 1) / kTwFine + 1;
  for (int h = threadIdx.x; h < nc; h += T) stw[kTwFinePadded + h] = __ldg(p.tw + h * kTwFine);
}

__device__ __forceinline__ float2 tw_lookup(const float2* stw, int k) {
  return cmul(stw[kTwFinePadded + (k >> kTwFineShift)], stw[tw_fine_slot(k & (kTwFine - 1))]);
}

// x[t] *= w^(t*jt), t = 1..R-1: a table lookup for t = 1, 9, 17, ... and
// complex products with w^jt in between (at most 7 products per lookup, so
// the rounding stays within a few ulp); no twiddle array is kept.
template <int R>
__device__ __forceinline__ void apply_twiddles(const float2* stw, int jt, float2 (&x)[R]) {
  const float2 w1 = tw_lookup(stw, jt);
  float2 w = w1;
#pragma unroll
  for (int t = 1; t < R; ++t) {
    if (t > 1) w = ((t - 1) & 7) == 0 ? tw_lookup(stw, t * jt) : cmul(w, w1);
    x[t] = cmul(x[t], w);
  }
}

// Stage functions are out of line by default (one copy per radix, called
// through the ABI); a translation unit may define FXC_FFT_STAGE_ATTR before
// including this header to inline them instead.
#ifndef FXC_FFT_STAGE_ATTR
#define FXC_FFT_STAGE_ATTR __noinline__
#endif
#ifndef FXC_FFT_NL_ATTR
#define FXC_FFT_NL_ATTR __noinline__
#endif

template <int R, int T, bool DIT>
__device__ FXC_FFT_STAGE_ATTR void fft_stage_ip(float2* buf, int n, int L, uint32_t m, const float2* stw,
                                                int tw_step, bool conj_in, bool conj_out) {
  const int nb = n / R;
  const int B = L * R;
  // b / L by a multiply-high with m = fft_lmag(L) (exact for b, L below
  // 2^16 as here); L == 1 has no twiddles
  for (int b = threadIdx.x; b < nb; b += T) {
    const int blk = L > 1 ? (int)__umulhi((uint32_t)b, m) : b;
    const int j = b - blk * L;
    const int base = blk * B + j;
    float2 x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) {
      float2 e = buf[base + t * L];
      x[t] = conj_in ? conjf2(e) : e;
    }
    if (DIT && j != 0) apply_twiddles<R>(stw, j * tw_step, x);
    dft_any<R>(x);
    if (!DIT && j != 0) apply_twiddles<R>(stw, j * tw_step, x);
#pragma unroll
    for (int t = 0; t < R; ++t) buf[base + t * L] = conj_out ? conjf2(x[t]) : x[t];
  }
  __syncthreads();
}

// SMOOTH: the plan's radices are 2, 3, 4, 5, 7 and 8 only (the 7-smooth
// Bluestein lengths), so no other stage is instantiated (code size and
// compile time of the row kernels that carry both transform forms).
template <int T, bool DIT, bool COMP = true, bool SMOOTH = false>
__device__ __forceinline__ void fft_run_stage(float2* buf, const FftPlan& p, const float2* stw,
                                              int R, int L, uint32_t m, int tw_step, bool ci, bool co) {
  if constexpr (SMOOTH) {
    switch (R) {
      case 2: fft_stage_ip<2, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
      case 4: fft_stage_ip<4, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
      case 8: fft_stage_ip<8, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
      case 3: fft_stage_ip<3, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
      case 5: fft_stage_ip<5, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
      case 7: fft_stage_ip<7, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
      default: break;  // any_plan picks 7-smooth Bluestein lengths
    }
    return;
  }
  if constexpr (COMP) {
    switch (R) {
      case 6: fft_stage_ip<6, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      case 9: fft_stage_ip<9, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      case 10: fft_stage_ip<10, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      case 12: fft_stage_ip<12, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      case 14: fft_stage_ip<14, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      case 15: fft_stage_ip<15, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      case 21: fft_stage_ip<21, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); return;
      default: break;
    }
  }
  switch (R) {
    case 2: fft_stage_ip<2, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 4: fft_stage_ip<4, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 8: fft_stage_ip<8, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 3: fft_stage_ip<3, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 5: fft_stage_ip<5, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 7: fft_stage_ip<7, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 11: fft_stage_ip<11, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 13: fft_stage_ip<13, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 17: fft_stage_ip<17, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 19: fft_stage_ip<19, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 23: fft_stage_ip<23, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 29: fft_stage_ip<29, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    case 31: fft_stage_ip<31, T, DIT>(buf, p.n, L, m, stw, tw_step, ci, co); break;
    default: break;  // rejected by fft_make_plan
  }
}

// Natural-order input, digit-reversed output. All T threads must call it
// after buf and the twiddle table stw (fft_twiddles_to_smem) are written and
// the CTA synchronised; the result is visible to the CTA on return.
template <int T, bool COMP = true, bool SMOOTH = false>
__device__ void fft_dif(float2* buf, const FftPlan& p, const float2* stw, bool inverse) {
  int L = p.n;
  int Rprod = 1;  // r_0 ... r_{s-1}
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    L /= R;
    // block length B = L*R = n / Rprod; twiddle w_B^{tj} = w_n^{t j Rprod}
    const int tw_step = Rprod * p.tw_stride;
    fft_run_stage<T, false, COMP, SMOOTH>(buf, p, stw, R, L, p.lmag[s], tw_step, inverse && s == 0,
                                          inverse && s == p.nstages - 1);
    Rprod *= R;
  }
}

// Digit-reversed input (the layout fft_dif produces), natural-order output.
template <int T, bool COMP = true, bool SMOOTH = false>
__device__ void fft_dit(float2* buf, const FftPlan& p, const float2* stw, bool inverse) {
  int L = 1;
  int Rprod = p.n;
  for (int s = p.nstages - 1; s >= 0; --s) {
    const int R = p.radix[s];
    Rprod /= R;
    const int tw_step = Rprod * p.tw_stride;
    fft_run_stage<T, true, COMP, SMOOTH>(buf, p, stw, R, L, p.lmag[s], tw_step, inverse && s == p.nstages - 1,
                                         inverse && s == 0);
    L *= R;
  }
}

// ---- pieces of a DIF transform whose input is formed on the fly and whose
// output is needed at a few frequencies only (the C2R + lag cut of the xc
// finalize) -----------------------------------------------------------------

// DIF stage 0 (one block of n points at stride L = n / R) with its inputs
// taken from load(k) instead of buf; buf then holds what fft_dif's stage 0
// leaves. load returns the butterfly input as is (any conjugation of an
// inverse transform already applied); it is a small value type (pointers
// and sizes), passed by value. These edge stages (this one and
// fft_dit_last_store_r) are out of line unless a translation unit defines
// FXC_FFT_EDGE_ATTR.
#ifndef FXC_FFT_EDGE_ATTR
#define FXC_FFT_EDGE_ATTR __noinline__
#endif

template <int R, int T, class Load>
__device__ FXC_FFT_EDGE_ATTR void fft_stage0_load_r(float2* buf, int L, const float2* stw, int tw_step, Load load) {
  for (int j = threadIdx.x; j < L; j += T) {
    float2 x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) x[t] = load(j + t * L);
    dft_any<R>(x);
    if (j != 0) apply_twiddles<R>(stw, j * tw_step, x);
#pragma unroll
    for (int t = 0; t < R; ++t) buf[j + t * L] = x[t];
  }
  __syncthreads();
}

// Stage 0 of a plan with at least two stages (stage 0 is then never the
// last, so no output conjugation applies).
template <int T, bool COMP = true, class Load>
__device__ __forceinline__ void fft_dif_stage0_load(float2* buf, const FftPlan& p, const float2* stw,
                                                    const Load& load) {
  const int R = p.radix[0];
  const int L = p.n / R;
  const int ts = p.tw_stride;
  if constexpr (COMP) {
    switch (R) {
      case 6: fft_stage0_load_r<6, T>(buf, L, stw, ts, load); return;
      case 9: fft_stage0_load_r<9, T>(buf, L, stw, ts, load); return;
      case 10: fft_stage0_load_r<10, T>(buf, L, stw, ts, load); return;
      case 12: fft_stage0_load_r<12, T>(buf, L, stw, ts, load); return;
      case 14: fft_stage0_load_r<14, T>(buf, L, stw, ts, load); return;
      case 15: fft_stage0_load_r<15, T>(buf, L, stw, ts, load); return;
      case 21: fft_stage0_load_r<21, T>(buf, L, stw, ts, load); return;
      default: break;
    }
  }
  switch (R) {
    case 2: fft_stage0_load_r<2, T>(buf, L, stw, ts, load); break;
    case 4: fft_stage0_load_r<4, T>(buf, L, stw, ts, load); break;
    case 8: fft_stage0_load_r<8, T>(buf, L, stw, ts, load); break;
    case 3: fft_stage0_load_r<3, T>(buf, L, stw, ts, load); break;
    case 5: fft_stage0_load_r<5, T>(buf, L, stw, ts, load); break;
    case 7: fft_stage0_load_r<7, T>(buf, L, stw, ts, load); break;
    case 11: fft_stage0_load_r<11, T>(buf, L, stw, ts, load); break;
    case 13: fft_stage0_load_r<13, T>(buf, L, stw, ts, load); break;
    case 17: fft_stage0_load_r<17, T>(buf, L, stw, ts, load); break;
    case 19: fft_stage0_load_r<19, T>(buf, L, stw, ts, load); break;
    case 23: fft_stage0_load_r<23, T>(buf, L, stw, ts, load); break;
    case 29: fft_stage0_load_r<29, T>(buf, L, stw, ts, load); break;
    case 31: fft_stage0_load_r<31, T>(buf, L, stw, ts, load); break;
    default: break;  // rejected by fft_make_plan
  }
}

// DIF stages [s0, s1) with neither input nor output conjugation (stages
// strictly between the first and the last of an inverse transform).
template <int T, bool COMP = true>
__device__ __forceinline__ void fft_dif_inner(float2* buf, const FftPlan& p, const float2* stw, int s0,
                                              int s1) {
  int L = p.n;
  int Rprod = 1;
  for (int s = 0; s < s1; ++s) {
    const int R = p.radix[s];
    L /= R;
    if (s >= s0) fft_run_stage<T, false, COMP>(buf, p, stw, R, L, p.lmag[s], Rprod * p.tw_stride, false, false);
    Rprod *= R;
  }
}

// The DIT stages but the last (stages nstages-1 .. 1; the inverse's input
// conjugation at the first of them): with fft_dit_last_store after it, the
// same transform as fft_dit.
// s_top < nstages - 1 starts below the top stage (run elsewhere, e.g. by
// fft_dit_first_load, with the input conjugation).
template <int T, bool COMP = true>
__device__ __forceinline__ void fft_dit_head(float2* buf, const FftPlan& p, const float2* stw, bool inverse,
                                             int s_top = -1) {
  if (s_top < 0) s_top = p.nstages - 1;
  int L = 1;
  int Rprod = p.n;
  for (int s = p.nstages - 1; s >= 1; --s) {
    const int R = p.radix[s];
    Rprod /= R;
    if (s <= s_top)
      fft_run_stage<T, true, COMP>(buf, p, stw, R, L, p.lmag[s], Rprod * p.tw_stride,
                                   inverse && s == p.nstages - 1, false);
    L *= R;
  }
}

// The first DIT stage (stage nstages-1: blocks of R adjacent points, no
// twiddles) with its inputs taken from load(k) for the frequency k each
// point holds -- k = iperm[base] + t n / R for point base + t of a block --
// instead of from a digit-reversed copy in buf; the inverse's input
// conjugation applied here.
template <int R, int T, class Load>
__device__ FXC_FFT_EDGE_ATTR void fft_dit_first_load_r(float2* buf, int nb, const int* __restrict__ iperm,
                                                       bool conj_in, bool conj_out, Load load) {
  for (int b = threadIdx.x; b < nb; b += T) {
    const int base = b * R;
    const int k0 = __ldg(iperm + base);
    float2 x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) {
      const float2 e = load(k0 + t * nb);
      x[t] = conj_in ? conjf2(e) : e;
    }
    dft_any<R>(x);
#pragma unroll
    for (int t = 0; t < R; ++t) buf[base + t] = conj_out ? conjf2(x[t]) : x[t];
  }
  __syncthreads();
}

template <int T, bool COMP = true, class Load>
__device__ __forceinline__ void fft_dit_first_load(float2* buf, const FftPlan& p, const int* iperm, bool inverse,
                                                   const Load& load) {
  const int R = p.radix[p.nstages - 1];
  const int nb = p.n / R;
  const bool ci = inverse, co = inverse && p.nstages == 1;
  if constexpr (COMP) {
    switch (R) {
      case 6: fft_dit_first_load_r<6, T>(buf, nb, iperm, ci, co, load); return;
      case 9: fft_dit_first_load_r<9, T>(buf, nb, iperm, ci, co, load); return;
      case 10: fft_dit_first_load_r<10, T>(buf, nb, iperm, ci, co, load); return;
      case 12: fft_dit_first_load_r<12, T>(buf, nb, iperm, ci, co, load); return;
      case 14: fft_dit_first_load_r<14, T>(buf, nb, iperm, ci, co, load); return;
      case 15: fft_dit_first_load_r<15, T>(buf, nb, iperm, ci, co, load); return;
      case 21: fft_dit_first_load_r<21, T>(buf, nb, iperm, ci, co, load); return;
      default: break;
    }
  }
  switch (R) {
    case 2: fft_dit_first_load_r<2, T>(buf, nb, iperm, ci, co, load); break;
    case 4: fft_dit_first_load_r<4, T>(buf, nb, iperm, ci, co, load); break;
    case 8: fft_dit_first_load_r<8, T>(buf, nb, iperm, ci, co, load); break;
    case 3: fft_dit_first_load_r<3, T>(buf, nb, iperm, ci, co, load); break;
    case 5: fft_dit_first_load_r<5, T>(buf, nb, iperm, ci, co, load); break;
    case 7: fft_dit_first_load_r<7, T>(buf, nb, iperm, ci, co, load); break;
    case 11: fft_dit_first_load_r<11, T>(buf, nb, iperm, ci, co, load); break;
    case 13: fft_dit_first_load_r<13, T>(buf, nb, iperm, ci, co, load); break;
    case 17: fft_dit_first_load_r<17, T>(buf, nb, iperm, ci, co, load); break;
    case 19: fft_dit_first_load_r<19, T>(buf, nb, iperm, ci, co, load); break;
    case 23: fft_dit_first_load_r<23, T>(buf, nb, iperm, ci, co, load); break;
    case 29: fft_dit_first_load_r<29, T>(buf, nb, iperm, ci, co, load); break;
    case 31: fft_dit_first_load_r<31, T>(buf, nb, iperm, ci, co, load); break;
    default: break;  // rejected by fft_make_plan
  }
}

// The last DIT stage (stage 0: one block at stride L = n / R, twiddles
// before the DFT) with each output handed to store(k, y) at its natural-order
// point k instead of written back to buf; a point is stored by one thread
// only. No barrier at the end: buf is still being read until the caller
// synchronises.
template <int R, int T, class Store>
__device__ FXC_FFT_EDGE_ATTR void fft_dit_last_store_r(const float2* buf, int L, const float2* stw, int tw_step,
                                                        bool conj_in, bool conj_out, Store store) {
  for (int j = threadIdx.x; j < L; j += T) {
    float2 x[R];
#pragma unroll
    for (int t = 0; t < R; ++t) {
      const float2 e = buf[j + t * L];
      x[t] = conj_in ? conjf2(e) : e;
    }
    if (j != 0) apply_twiddles<R>(stw, j * tw_step, x);
    dft_any<R>(x);
#pragma unroll
    for (int t = 0; t < R; ++t) store(j + t * L, conj_out ? conjf2(x[t]) : x[t]);
  }
}

template <int T, bool COMP = true, class Store>
__device__ __forceinline__ void fft_dit_last_store(const float2* buf, const FftPlan& p, const float2* stw,
                                                   bool inverse, const Store& store) {
  const int R = p.radix[0];
  const int L = p.n / R;
  const int ts = p.tw_stride;
  const bool ci = inverse && p.nstages == 1, co = inverse;
  if constexpr (COMP) {
    switch (R) {
      case 6: fft_dit_last_store_r<6, T>(buf, L, stw, ts, ci, co, store); return;
      case 9: fft_dit_last_store_r<9, T>(buf, L, stw, ts, ci, co, store); return;
      case 10: fft_dit_last_store_r<10, T>(buf, L, stw, ts, ci, co, store); return;
      case 12: fft_dit_last_store_r<12, T>(buf, L, stw, ts, ci, co, store); return;
      case 14: fft_dit_last_store_r<14, T>(buf, L, stw, ts, ci, co, store); return;
      case 15: fft_dit_last_store_r<15, T>(buf, L, stw, ts, ci, co, store); return;
      case 21: fft_dit_last_store_r<21, T>(buf, L, stw, ts, ci, co, store); return;
      default: break;
    }
  }
  switch (R) {
    case 2: fft_dit_last_store_r<2, T>(buf, L, stw, ts, ci, co, store); break;
    case 4: fft_dit_last_store_r<4, T>(buf, L, stw, ts, ci, co, store); break;
    case 8: fft_dit_last_store_r<8, T>(buf, L, stw, ts, ci, co, store); break;
    case 3: fft_dit_last_store_r<3, T>(buf, L, stw, ts, ci, co, store); break;
    case 5: fft_dit_last_store_r<5, T>(buf, L, stw, ts, ci, co, store); break;
    case 7: fft_dit_last_store_r<7, T>(buf, L, stw, ts, ci, co, store); break;
    case 11: fft_dit_last_store_r<11, T>(buf, L, stw, ts, ci, co, store); break;
    case 13: fft_dit_last_store_r<13, T>(buf, L, stw, ts, ci, co, store); break;
    case 17: fft_dit_last_store_r<17, T>(buf, L, stw, ts, ci, co, store); break;
    case 19: fft_dit_last_store_r<19, T>(buf, L, stw, ts, ci, co, store); break;
    case 23: fft_dit_last_store_r<23, T>(buf, L, stw, ts, ci, co, store); break;
    case 29: fft_dit_last_store_r<29, T>(buf, L, stw, ts, ci, co, store); break;
    case 31: fft_dit_last_store_r<31, T>(buf, L, stw, ts, ci, co, store); break;
    default: break;  // rejected by fft_make_plan
  }
}

// Frequency k of the DIF result, from buf as it stands before the last
// stage (blocks of R = radix[S-1] adjacent points, no twiddles in that
// stage): k's last digit t = k / (n / R) picks the butterfly output
//   sum_u buf[base + u] w_R^{t u},  base = perm[k] - t,
// with w_R^v read from the twiddle table as w_n^{v n / R} (and advanced by
// multiplication between table reads, as apply_twiddles does).
__device__ __forceinline__ float2 fft_dif_last_point(const float2* buf, const FftPlan& p, const float2* stw,
                                                     int k) {
  const int R = p.radix[p.nstages - 1];
  const int nr = p.n / R;
  const int t = k / nr;
  const int base = __ldg(p.perm + k) - t;
  float2 acc = buf[base];
  if (t == 0) {
    for (int u = 1; u < R; ++u) acc = cadd(acc, buf[base + u]);
    return acc;
  }
  const int step = nr * p.tw_stride;
  const float2 w1 = tw_lookup(stw, t * step);
  float2 w = w1;
  int v = t;  // t u mod R
  for (int u = 1; u < R; ++u) {
    if (u > 1) {
      v += t;
      if (v >= R) v -= R;
      w = ((u - 1) & 7) == 0 ? tw_lookup(stw, v * step) : cmul(w, w1);
    }
    acc = cadd(acc, cmul(buf[base + u], w));
  }
  return acc;
}

// Position of natural-order frequency k in the digit-reversed layout:
// k = d_0 + r_0 d_1 + r_0 r_1 d_2 + ...  ->  pos = d_0 L_0 + d_1 L_1 + ...
__host__ __device__ inline int fft_digit_pos(const FftPlan& p, int k) {
  int pos = 0;
  int L = p.n;
  for (int s = 0; s < p.nstages; ++s) {
    const int R = p.radix[s];
    L /= R;
    const int d = k % R;
    k /= R;
    pos += d * L;
  }
  return pos;
}

// Transform entry points whose linkage a translation unit chooses
// (FXC_FFT_NL_ATTR: out of line by default, so that the caller's live values
// stay out of the stage loops' registers; the sac2spec row kernels define it
// inline, which measured faster there).
template <int T, bool COMP = true>
__device__ FXC_FFT_NL_ATTR void fft_dif_nl(float2* buf, const FftPlan& p, const float2* stw, bool inverse) {
  fft_dif<T, COMP>(buf, p, stw, inverse);
}
template <int T, bool COMP = true>
__device__ FXC_FFT_NL_ATTR void fft_dit_nl(float2* buf, const FftPlan& p, const float2* stw, bool inverse) {
  fft_dit<T, COMP>(buf, p, stw, inverse);
}

}  // namespace fxc
