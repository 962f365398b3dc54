/*
 * fastxc_gb300 -- C ABI of the GB300 (sm_103a) ambient-noise correlation
 * library.
 *
 * The reference (wangkingh/FastXC) has no library ABI: its boundary is
 * "Python builds an argv string -> native executable -> files + exit code"
 * (fastxc/runtime/command_runner.py:97-210). This header is the thin library
 * that sits under drop-in replacements for those executables. Every entry
 * point below names the reference function or kernel whose behaviour it
 * reproduces.
 *
 * Conventions
 *   - Every function returns FXC_OK (0) or a negative FXC_ERR_* status; the
 *     message of the last failure on the calling thread is fxc_last_error().
 *     Nothing in the library calls exit().
 *   - Complex arrays are interleaved float pairs (re, im), the layout of
 *     cuComplex / numpy complex64. Pitches of complex arrays count complex
 *     elements; pitches of real arrays count floats.
 *   - "d_" pointers are device pointers on the context's device; "h_"
 *     pointers are host pointers (pinned memory gives full copy speed,
 *     pageable memory works).
 *   - Work is enqueued on the context's stream; functions return once the
 *     work is enqueued unless documented as synchronous (the *_host calls).
 *   - A context is used by one thread at a time; distinct contexts may be
 *     used concurrently.
 */
#ifndef FASTXC_GB300_H
#define FASTXC_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FXC_OK 0
#define FXC_ERR_INVALID (-1)     /* bad argument or shape */
#define FXC_ERR_CUDA (-2)        /* CUDA runtime error (message has the name) */
#define FXC_ERR_UNSUPPORTED (-3) /* transform length / shape not supported */
#define FXC_ERR_NOMEM (-4)       /* device or host allocation failed */
#define FXC_ERR_IO (-5)          /* file format or I/O error */
#define FXC_ERR_NODEVICE (-6)    /* no CUDA device / driver */
#define FXC_ERR_TIMEOUT (-7)     /* a kernel's bounded device-side wait gave up */
#define FXC_ERR_NOTFOUND (-8)    /* an input file or folder does not exist */

#define FXC_XC_PLAIN 0  /* FP32 CUDA-core per-pair product, register blocked */
#define FXC_XC_TENSOR 1 /* BF16 hi/lo split tcgen05 contraction S(f)=Y^H Y */
/* layouts of the tensor contraction (fxc_pairplan_set_layout) */
#define FXC_XC_LAYOUT_AUTO 0      /* whole-bin unless a short contraction over <= 128 channels */
#define FXC_XC_LAYOUT_WHOLE_BIN 1 /* one CTA per bin over every tile (<= 192 channels, one tile layer) */
#define FXC_XC_LAYOUT_TILED 2     /* persistent CTAs over (tile, bin) items */

typedef struct fxc_ctx fxc_ctx;
typedef struct fxc_pairplan fxc_pairplan;

/* ---- library / context --------------------------------------------------- */

/* Message of the last failure on this thread ("" when none). */
const char *fxc_last_error(void);
/* ABI version: major*10000 + minor*100 + patch. */
int fxc_version(void);
/* Number of kernel launches the library made on this thread since the last
 * reset; lets callers attribute device work to the library. */
int64_t fxc_launch_count(void);
void fxc_launch_count_reset(void);

/* Per-kernel device timing (a measurement aid with no counterpart in the
 * reference). While enabled on a context, the library brackets the launches
 * of its dominant kernels (currently the tensor-core contraction,
 * "k_xc_tc_gemm_bin" / "k_xc_tc_gemm") with CUDA events on the context
 * stream. fxc_ctx_kernel_time synchronises that stream, returns the summed
 * event time and launch count of the named kernel since the last query and
 * forgets them. Disabling drops every pending record. */
int fxc_ctx_kernel_timing(fxc_ctx *ctx, int enable);
int fxc_ctx_kernel_time(fxc_ctx *ctx, const char *kernel, double *total_ms, int64_t *launches);
/* Phases of the last fxc_xc_run_host on this context that ran while kernel
 * timing was enabled, from CUDA events on its two streams (ms): [0] total,
 * [1] copy stream busy with host-to-device copies, [2] end of the last
 * host-to-device copy, [3] compute busy on the chunks, [4] tail after the
 * last host-to-device copy, [5] finalize + device-to-host copies. Entries
 * not measured are -1. Writes min(n, 6) values (the rest -1). */
int fxc_ctx_host_phases(fxc_ctx *ctx, double *out_ms, int32_t n);

/* Create a context bound to `device`. `stream` is a cudaStream_t (NULL = the
 * legacy default stream). The context owns its scratch buffers and FFT
 * tables. */
int fxc_ctx_create(int device, void *stream, fxc_ctx **out);
int fxc_ctx_destroy(fxc_ctx *ctx);
int fxc_ctx_set_stream(fxc_ctx *ctx, void *stream);
int fxc_ctx_synchronize(fxc_ctx *ctx);

/* CUDA-graph capture of a launch sequence (no counterpart in the reference,
 * which launches every kernel from the host each time). Between
 * fxc_graph_begin and fxc_graph_end, calls on the context are recorded
 * instead of run; fxc_graph_launch replays them on the context's stream
 * with the same pointers and sizes. Only device-resident calls that neither
 * synchronise nor allocate can be recorded: fxc_xc_pack,
 * fxc_xc_stack_packed, fxc_xc_stack, fxc_xc_finalize and
 * fxc_xc_stack_finalize_packed after one uncaptured call of the same shapes
 * (which sizes the context's scratch and FFT tables). The context must use a
 * non-default stream. fxc_graph_end fails with FXC_ERR_CUDA when a recorded
 * call synchronised or allocated. */
typedef struct fxc_graph fxc_graph;
int fxc_graph_begin(fxc_ctx *ctx);
int fxc_graph_end(fxc_ctx *ctx, fxc_graph **out);
int fxc_graph_launch(fxc_ctx *ctx, const fxc_graph *g);
int fxc_graph_destroy(fxc_graph *g);

/* ---- memory helpers ------------------------------------------------------
 * For callers without a CUDA runtime of their own (the drop-in executables,
 * ctypes). No reference counterpart: the reference executables call
 * cudaMalloc / cudaMemcpy directly. fxc_memcpy is asynchronous on the
 * context's stream (kind: FXC_COPY_H2D, FXC_COPY_D2H, FXC_COPY_D2D);
 * fxc_device_free synchronises the stream first. */
#define FXC_COPY_H2D 1
#define FXC_COPY_D2H 2
#define FXC_COPY_D2D 3
int fxc_device_alloc(fxc_ctx *ctx, size_t bytes, void **out);
int fxc_device_free(fxc_ctx *ctx, void *ptr);
int fxc_host_alloc(size_t bytes, void **out);
int fxc_host_free(void *ptr);
int fxc_memcpy(fxc_ctx *ctx, void *dst, const void *src, size_t bytes, int kind);

/* ---- FFT (replaces every cuFFT plan of the reference's hot path) --------- */

/* Batched complex transform of length n, unnormalised (cuFFT convention:
 * forward exp(-2 pi i jk/n), inverse exp(+2 pi i jk/n)). Row r of the input
 * starts at d_in + 2*r*in_pitch floats. In-place is allowed. */
int fxc_fft_c2c(fxc_ctx *ctx, const float *d_in, float *d_out, int n, int batch,
                int64_t in_pitch, int64_t out_pitch, int inverse);
/* Batched real-to-complex transform: n reals -> n/2+1 complex bins
 * (cufftExecR2C). */
int fxc_fft_r2c(fxc_ctx *ctx, const float *d_in, float *d_out, int n, int batch,
                int64_t in_pitch, int64_t out_pitch);
/* Batched complex-to-real transform: n/2+1 bins -> n reals, unnormalised
 * (cufftExecC2R; the imaginary parts of the DC and Nyquist bins are
 * ignored). n must be even. */
int fxc_fft_c2r(fxc_ctx *ctx, const float *d_in, float *d_out, int n, int batch,
                int64_t in_pitch, int64_t out_pitch);
/* 1 if the length is supported by the fused in-CTA transforms. */
int fxc_fft_supported(int n, int real_transform);

/* ---- sac2spec: windows -> normalised, whitened output spectra ----------- */

#define FXC_S2S_MAX_BANDS 100 /* MAXBAND, native/sac2spec/include/config.h:8 */

/* Whitening codes (-W a/...) and normalisation codes (-N) of the sac2spec
 * command line (native/sac2spec/include/config.h:16-27). */
#define FXC_WHITEN_NONE 0
#define FXC_WHITEN_BEFORE 1
#define FXC_WHITEN_AFTER 2
#define FXC_WHITEN_BOTH 3
#define FXC_NORM_NONE 0
#define FXC_NORM_RUNABS_MF 1
#define FXC_NORM_ONEBIT 2
#define FXC_NORM_RUNABS 3

typedef struct fxc_s2s_plan {
  float delta;
  int32_t npts;          /* llround(sac_len / delta) */
  int32_t segment_pts;   /* segment_length_from_seconds (fft_length.c:90-108) */
  int32_t shift_pts;
  int32_t nstep;         /* (npts - seg) / shift + 1 */
  int32_t output_nfft;   /* next even 2357-smooth >= seg + lag samples, <= 2 seg */
  int32_t nspec;         /* output_nfft / 2 + 1 */
  int32_t filter_padding;
  int32_t filter_nfft;
  float freq_low, freq_high; /* broad band (first filter) */
  int32_t f_idx1, f_idx2, f_idx3, f_idx4; /* whitening band taper bins */
  int32_t taper_pts;     /* (int)(2 / f_low / delta) */
  int32_t runabs_win;    /* 2 * int(1 / (0.667 f_low * delta)) + 1 */
  int32_t whiten_win;    /* int(0.02 * seg * delta) */
  int32_t whiten, normalize, phase_only;
  int32_t nfilters;
  float band_freq_low[FXC_S2S_MAX_BANDS];
} fxc_s2s_plan;

/* Segment / FFT / band planning of sac2spec (native/sac2spec/cuda.main.cu:
 * 203-296, fft_length.c:39-108, core/filter_response.c:74-104). Filters are
 * the filter.txt entries (first = broad band): b and a are [nfilters][5]. */
int fxc_s2s_plan_init(float sac_len, float win_len, float shift_len, float xcorr_lag, float delta,
                      const double *h_b, const double *h_a, const float *h_freq_low,
                      const float *h_freq_high, int32_t nfilters, int32_t whiten,
                      int32_t normalize, int32_t phase_only, fxc_s2s_plan *out);
/* Zero-phase power responses |B/A|^2 on filter_nfft/2+1 bins, float
 * (calFilterPowerResp, core/filter_response.c:186-233); h_out is
 * [nfilters][filter_nfft/2+1]. */
int fxc_s2s_filter_response(const fxc_s2s_plan *plan, const double *h_b, const double *h_a,
                            int32_t nfilters, float *h_out);
/* ComputeWorkerBatch (native/sac2spec/worker/compute.cu:8-272) for nsteps
 * windows (h_steps: window indices < nstep) of nrows channel series.
 * d_series is [nrows][series_pitch] float with series_len valid samples
 * (shorter series are zero-padded as read_sac_buffer does); rows are grouped
 * by station, num_ch consecutive rows per station. d_responses is the
 * device copy of fxc_s2s_filter_response's output. d_out receives
 * [nsteps][nrows][out_pitch] complex spectra (nspec bins used). */
int fxc_s2s_run(fxc_ctx *ctx, const fxc_s2s_plan *plan, const float *d_series,
                int64_t series_pitch, int64_t series_len, int32_t nrows, int32_t num_ch,
                const int32_t *h_steps, int32_t nsteps, const float *d_responses, float *d_out,
                int64_t out_pitch);

/* ---- xc_fast: correlation + within-window linear stack ------------------ */

typedef struct fxc_xc_shape {
  int32_t nspec;   /* spectrum bins per window (output_nfft/2+1) */
  int32_t nstep;   /* windows per timestamp */
  int32_t nfft;    /* 2*(nspec-1) */
  int32_t half_cc; /* llround(cc_length/dt), capped at nspec-1 */
  int32_t cc_size; /* 2*half_cc+1 */
  float dt;
} fxc_xc_shape;

/* finalize_shape (native/xc/io/input.cu:1033-1054). */
int fxc_xc_shape_init(int32_t nspec, int32_t nstep, float dt, float cc_length,
                      fxc_xc_shape *out);

/* Build a correlation plan for the pair list (src[p], rec[p]) over channel
 * indices in [0, nchan). The list order is the output order (the order of
 * the reference's XcTask list, native/xc/worker/scheduler.cu:65-167). The
 * plan groups pairs into register tiles of up to 16 x 16 channels. Host
 * arrays; the plan uploads what the kernels need. */
int fxc_pairplan_create(fxc_ctx *ctx, const int32_t *h_src, const int32_t *h_rec, int64_t npairs,
                        int32_t nchan, fxc_pairplan **out);
int fxc_pairplan_destroy(fxc_pairplan *plan);
int64_t fxc_pairplan_npairs(const fxc_pairplan *plan);
int64_t fxc_pairplan_ntiles(const fxc_pairplan *plan);

/* stack[p, f] = scale * sum_w conj(Y[w, src_p, f]) * Y[w, rec_p, f]
 * for f < nspec. d_spec is [nwin][nchan][spec_pitch] complex (the stepack
 * payload layout, native/sac2spec/io/stepack_writer.c); d_stack is
 * [npairs][stack_pitch] complex. Optional d_mask (NULL = none) is
 * [nwin][nchan] uint8: a window with mask 0 contributes exactly zero.
 * Replaces the nstep launches of accumulateStepXc2DKernel
 * (native/xc/kernels/cuda.kernels.cu:16-36, loop at
 * native/xc/worker/async_workers.cu:66-83). */
int fxc_xc_stack(fxc_ctx *ctx, const fxc_pairplan *plan, const float *d_spec, int64_t nwin,
                 int32_t nchan, int32_t nspec, int64_t spec_pitch, const uint8_t *d_mask,
                 float scale, float *d_stack, int64_t stack_pitch, int method);

/* Tensor-core operand form of the spectra: per bin, bf16 hi/lo planes of
 * the real and imaginary parts laid out as UMMA core-matrix tiles. Packing
 * once and keeping the result resident lets many pair plans (requests)
 * correlate the same spectra without repacking. fxc_xc_stack with
 * FXC_XC_TENSOR is fxc_xc_pack + fxc_xc_stack_packed through context
 * scratch. Same stacked-spectrum contract as accumulateStepXc2DKernel
 * (native/xc/kernels/cuda.kernels.cu:16-36). */
int fxc_xc_packed_bytes(int32_t nchan, int64_t nwin, int32_t nspec, int64_t *out_bytes);
int fxc_xc_pack(fxc_ctx *ctx, const float *d_spec, int64_t nwin, int32_t nchan, int32_t nspec,
                int64_t spec_pitch, const uint8_t *d_mask, void *d_packed);
int fxc_xc_stack_packed(fxc_ctx *ctx, const fxc_pairplan *plan, const void *d_packed, int64_t nwin,
                        int32_t nspec, float scale, float *d_stack, int64_t stack_pitch);
/* fxc_xc_stack_packed + fxc_xc_finalize in one call, the stack in context
 * scratch (accumulateStepXc2DKernel loop + finalize_xc_batch,
 * native/xc/worker/async_workers.cu:66-83, executor.cu:6-55): d_ncf is
 * [npairs][cc_size]. */
int fxc_xc_stack_finalize_packed(fxc_ctx *ctx, const fxc_pairplan *plan, const void *d_packed, int64_t nwin,
                                 int32_t nspec, float scale, const fxc_xc_shape *shape, float *d_ncf);

/* ncf[p, j] = C2R(stack[p] * (-1)^f)[nfft/2 - half_cc + j] / (nfft * dt),
 * j < cc_size. d_ncf is [npairs][cc_size] float. Replaces
 * finalize_xc_batch (native/xc/worker/executor.cu:6-55). */
int fxc_xc_finalize(fxc_ctx *ctx, const float *d_stack, int64_t npairs, int64_t stack_pitch,
                    const fxc_xc_shape *shape, float *d_ncf);

/* fxc_xc_stack + fxc_xc_finalize with the stack in context scratch memory.
 * scale is normally 1/nstep (async_workers.cu:66). */
int fxc_xc_run(fxc_ctx *ctx, const fxc_pairplan *plan, const float *d_spec, int64_t nwin,
               int32_t nchan, int64_t spec_pitch, const uint8_t *d_mask, float scale,
               const fxc_xc_shape *shape, float *d_ncf, int method);

/* Host-buffer variant of fxc_xc_run: copies h_spec ([nwin][nchan][spec_pitch]
 * complex) to the device, runs, copies the NCFs back to h_ncf
 * ([npairs][cc_size]) and synchronises. The windows travel in 64-window
 * chunks that are stacked as they land (FXC_XC_TENSOR: each chunk packed and
 * contracted, accumulated into the stack through the bin-major transpose),
 * so the FP32 summation order differs from fxc_xc_run's at the chunk
 * boundaries. */
int fxc_xc_run_host(fxc_ctx *ctx, const fxc_pairplan *plan, const float *h_spec, int64_t nwin,
                    int32_t nchan, int64_t spec_pitch, const uint8_t *h_mask, float scale,
                    const fxc_xc_shape *shape, float *h_ncf, int method);

/* ---- ENZ -> RTZ rotation of nine-component NCFs ------------------------- */

/* The 9 x 9 float32 matrix of build_rotate_matrix
 * (fastxc/operators/rotation/python_rotate.py:33-95), row-major: rows R-R,
 * R-T, R-Z, T-R, T-T, T-Z, Z-R, Z-T, Z-Z; columns E-E, E-N, E-Z, N-E, N-N,
 * N-Z, Z-E, Z-N, Z-Z. Host function (no device work). */
int fxc_rotate_matrix(double azimuth_deg, double back_azimuth_deg, float *out81);

/* d_rtz[p][r][t] = sum_c d_mats[p][r][c] * d_enz[p][c][t] for npairs pairs
 * of nine traces ([npairs][9][pitch] float32, npts samples used) --
 * rotate_enz_to_rtz (python_rotate.py:98-105) batched over pairs. */
int fxc_rotate_enz_rtz(fxc_ctx *ctx, const float *d_enz, int64_t npairs, int32_t npts, int64_t pitch,
                       const float *d_mats, float *d_rtz);

/* Cross-day fold of complex stack rows (no counterpart in the reference,
 * whose linear stack averages finished per-day NCF files):
 * d_dst[h_dst_idx[r]][c] += d_src[h_src_idx[r]][c] (or = with assign != 0,
 * for rows that start a group) for r < nrows and c < ncols complex columns;
 * pitches in complex elements; destination rows distinct within a call and
 * < dst_rows, source rows < src_rows. One call per timestamp builds the sum
 * over timestamps of per-timestamp stacks, from which one finalize gives
 * the mean of the per-timestamp NCFs that _linear_stack_group
 * (fastxc/operators/stacking/linear_stack.py:228-247) computes, because the
 * finalize is linear. Synchronises the context stream. */
int fxc_xc_rows_accumulate(fxc_ctx *ctx, const float *d_src, int64_t src_rows, int64_t src_pitch,
                           const int64_t *h_src_idx, const int64_t *h_dst_idx, int64_t nrows, float *d_dst,
                           int64_t dst_rows, int64_t dst_pitch, int32_t ncols, int32_t assign);

/* ---- stacking: linear stack, PWS, TF-PWS -------------------------------- */

/* Cross-timestamp linear stack (_linear_stack_group,
 * fastxc/operators/stacking/linear_stack.py:228-247): out[p] = float(sum of
 * double(trace) / count) over traces [h_offsets[p], h_offsets[p]+h_counts[p])
 * of d_traces ([*][nsamples]). Bit-identical to the reference's sequential
 * FP64 sum: the sum is formed exactly in int64 fixed point where that
 * provably equals the FP64 sequence, and by the FP64 loop elsewhere (NaN,
 * infinities, terms too small beside the largest). At most 65535 pairs per
 * call (FXC_ERR_INVALID above). */
int fxc_linear_stack(fxc_ctx *ctx, const float *d_traces, const int64_t *h_offsets,
                     const int32_t *h_counts, int32_t npairs, int32_t nsamples, float *d_out);

/* Substack prestacking of each pair's traces into groups of `substack`
 * (< 2 -> 1): mode 0 group means with weight count/num_segments and
 * linear = sum(mean*weight) (prepare_sourcepack_host_item,
 * native/pws/io/sourcepack_io.cu:385-478); mode 1 group sums with weight
 * count/num_segments and linear = sum(sum)/num_segments (native/tfpws/io/
 * sourcepack_io.cu:440-490). Writes h_group_offsets/h_group_counts
 * ([npairs]) on the host, d_groups [total_groups][nsamples], d_weights
 * [total_groups], d_linear [npairs][nsamples]. Synchronous. */
int fxc_stack_prestack(fxc_ctx *ctx, const float *d_traces, const int64_t *h_trace_offsets,
                       const int32_t *h_trace_counts, int32_t npairs, int32_t nsamples,
                       int32_t substack, int32_t mode, float *d_groups, float *d_weights,
                       float *d_linear, int64_t *h_group_offsets, int32_t *h_group_counts);

/* Phase-weighted stack (compute_pws_host_batch, native/pws/worker/gpu.cu:
 * 87-282): analytic signal of every group, unit phasors (modulus floor
 * 1e-7), weighted mean, out = linear * |mean|^power (power 1 in the
 * reference). Synchronous. */
int fxc_pws_run(fxc_ctx *ctx, const float *d_groups, const float *d_weights,
                const int64_t *h_group_offsets, const int32_t *h_group_counts, int32_t npairs,
                const float *d_linear, int32_t nsamples, float power, float *d_out);

/* Streaming PWS for groups that arrive one at a time (one day's NCF of
 * every pair per call): d_acc ([npairs][nsamples] complex) and d_lin
 * ([npairs][nsamples]) start zeroed; each add accumulates weight x the unit
 * analytic phasor (modulus floor 1e-7) of row p of d_rows (row pitch
 * rows_pitch floats) into d_acc and weight x the row into d_lin; finish
 * writes out = lin * |acc|^power. With weight 1/G over G groups this is
 * fxc_stack_prestack (substack 1) + fxc_pws_run without holding the G
 * groups. Asynchronous on the context's stream. No reference counterpart
 * (the reference stacks whole SourcePack groups). */
int fxc_pws_stream_add(fxc_ctx *ctx, const float *d_rows, int64_t rows_pitch, int32_t npairs, int32_t nsamples,
                       float weight, float *d_acc, float *d_lin);
int fxc_pws_stream_finish(fxc_ctx *ctx, const float *d_acc, const float *d_lin, int32_t npairs, int32_t nsamples,
                          float power, float *d_out);

/* S-transform time-frequency PWS (compute_tfpws_from_prestack,
 * native/tfpws/core/tfpws_compute.cu:19-366): for every frequency of the
 * nsamples/2+1 bins the Gaussian voices (scale 0.1) of the groups and of
 * the linear stack, the phase weight, the weighted voice summed over time;
 * optional -F band blend (taper_hz < 0 -> 5% of the band); final inverse,
 * real part / N. Synchronous. */
int fxc_tfpws_run(fxc_ctx *ctx, const float *d_groups, const float *d_weights,
                  const int64_t *h_group_offsets, const int32_t *h_group_counts, int32_t npairs,
                  const float *d_linear, int32_t nsamples, float delta, int32_t band_limited,
                  float fmin, float fmax, float taper_hz, float power, float *d_out);

/* Autotuner of the stack method and contraction layout: times the plain
 * FP32 kernel (16 x 16 channel tiles) and the tcgen05 BF16 hi/lo
 * contraction (pack + 128 x N tiles) in each layout the plan admits (whole
 * bin: one CTA per bin over every tile; tiled: persistent CTAs over (tile,
 * bin) items) on the first min(nspec, 512) bins of d_spec. Returns the
 * faster method in *method (FXC_XC_PLAIN / FXC_XC_TENSOR) with the sample
 * times (ms, -1 when a candidate does not apply; ms_* may be null;
 * *ms_tensor is the faster layout's), and sets the plan's contraction
 * layout to the faster one. Decisions are cached per (device, channels,
 * windows, pairs, tiles) for the process. Must not overlap a run of the
 * same plan. No reference counterpart (the reference has one kernel).
 * Synchronous. */
int fxc_xc_autotune(fxc_ctx *ctx, const fxc_pairplan *plan, const float *d_spec, int64_t nwin, int32_t nchan,
                    int32_t nspec, int64_t spec_pitch, int32_t *method, float *ms_plain, float *ms_tensor);

/* fxc_xc_autotune with every candidate's time: *layout the faster tensor
 * layout (FXC_XC_LAYOUT_WHOLE_BIN / _TILED), ms[3] = plain, whole-bin,
 * tiled (-1 where a candidate does not apply; ms may be null). */
int fxc_xc_autotune_layout(fxc_ctx *ctx, const fxc_pairplan *plan, const float *d_spec, int64_t nwin,
                           int32_t nchan, int32_t nspec, int64_t spec_pitch, int32_t *method, int32_t *layout,
                           float *ms);

/* Contraction layout preference of a plan's tensor path (FXC_XC_LAYOUT_*),
 * honoured where the plan admits it (a whole-bin preference on a plan
 * without the whole-bin tile geometry runs tiled). For plans of pair
 * blocks that take a layout tuned on the whole pair list. */
int fxc_pairplan_set_layout(fxc_pairplan *plan, int32_t layout);

/* Layouts the plan admits, as a bit mask of 1 << FXC_XC_LAYOUT_* (0: no
 * tensor tiles), and the layout a run of nwin windows takes. */
int fxc_pairplan_layouts(const fxc_pairplan *plan, int64_t nwin, int32_t *admitted, int32_t *effective);

/* ---- serving: correlation jobs over resident station spectra ------------
 * No counterpart in the reference (its stages are batch executables). A
 * server owns one device, `slots` concurrent job slots (each a host thread,
 * a CUDA stream and a context), an HBM arena of station-day spectra
 * ([nstep][3 components][nspec] complex per station-day, LRU-evicted when
 * no running job holds them) and an HBM arena of job working memory. Queued
 * jobs are admitted first-fit by free working memory as slots free up (a job
 * older than max_wait_s is not overtaken); admitted jobs run concurrently.
 * A job: every cross-station component pair (9 per station pair, stations
 * in the given order, src = the earlier station) of `nsta` stations over
 * days [day0, day0 + ndays): the mean of the per-window cross spectra, the
 * +-lag NCF (fxc_xc_finalize), and with pws != 0 also a phase-weighted
 * stack of the per-day NCFs (fxc_pws_run, weight power pws_power). Spectra
 * geometry per delta follows the sac2spec planning of a day-long record
 * with win_len-second windows (shift = win_len) and lag_max. With
 * synthetic != 0 a missing station-day is generated from a seeded hash (a
 * pure function of seed, station, day, delta); otherwise it must be put
 * first. Results of a job depend only on the job and its spectra, not on
 * which other jobs run beside it. */
typedef struct fxc_server fxc_server;
typedef struct fxc_server_config {
  int32_t device;
  int32_t slots;        /* concurrent jobs */
  double cache_gib;     /* spectra arena */
  double work_gib;      /* job working-memory arena (admission budget) */
  double chunk_gib;     /* gathered spectra per stacking pass */
  int32_t synthetic;
  uint64_t seed;
  float win_len;        /* seconds */
  float lag_max;        /* seconds; largest lag a job may ask for */
  double max_wait_s;    /* <= 0: no anti-starvation bound */
  int32_t keep_results; /* copy NCFs to host memory for fxc_server_fetch */
} fxc_server_config;
typedef struct fxc_job {
  const int32_t *stations;
  int32_t nsta;
  int32_t day0, ndays;
  float delta;          /* sampling interval of the spectra, s */
  float lag;            /* NCF half length, s */
  int32_t method;       /* FXC_XC_PLAIN, FXC_XC_TENSOR, or -1: autotuned per job shape */
  int32_t pws;
  float pws_power;
} fxc_job;
typedef struct fxc_job_info {
  int64_t npairs, cc_size, nspec, pair_windows;
  double submit_s, start_s, end_s; /* host steady clock: queued, admitted, results on the host */
  int32_t status;
} fxc_job_info;
typedef struct fxc_server_stats_t {
  int64_t jobs_done, pair_windows, queued, cache_entries, cache_used_bytes, work_used_bytes;
} fxc_server_stats_t;
int fxc_server_create(const fxc_server_config *cfg, fxc_server **out);
int fxc_server_destroy(fxc_server *s);
/* nspec and windows per day of the spectra at this delta */
int fxc_server_geometry(fxc_server *s, float delta, int32_t *nspec, int32_t *nstep);
/* h_spec: [nstep][3][nspec] complex of one station-day */
int fxc_server_put_spectra(fxc_server *s, int32_t station, int32_t day, float delta, const float *h_spec);
int fxc_server_submit(fxc_server *s, const fxc_job *job, int64_t *job_id);
/* blocks until the job is done or failed, or timeout_s seconds passed
 * (timeout_s <= 0: no limit; FXC_ERR_TIMEOUT when it ran out or the server
 * is being destroyed) */
int fxc_server_wait(fxc_server *s, int64_t job_id, double timeout_s, fxc_job_info *info);
/* h_ncf / h_pws: [npairs][cc_size]; either may be null */
int fxc_server_fetch(fxc_server *s, int64_t job_id, float *h_ncf, float *h_pws);
int fxc_server_release(fxc_server *s, int64_t job_id);
int fxc_server_stats(fxc_server *s, fxc_server_stats_t *out);

/* ---- memory planners (host only, no GPU) ------------------------------------------ */

/* Device bytes one fxc_xc_run_host call over npairs pairs reserves (chunk
 * ring, mask, NCF staging, stacked spectra, pair tables; on the tensor path
 * also one chunk's packed operands and the bin-major rows). No counterpart
 * in the reference, whose own model is native/xc/memory/memory.cu:112-399. */
int fxc_xc_host_bytes(int64_t npairs, int64_t nwin, int32_t nchan, int64_t spec_pitch, const fxc_xc_shape *shape,
                      int method, int has_mask, int64_t *bytes);
/* Largest pair count per fxc_xc_run_host call whose bytes fit budget_bytes
 * (binary search over fxc_xc_host_bytes): the pair-block sizing of
 * native/xc/memory/memory.cu:277-399 for this library's buffers.
 * FXC_ERR_NOMEM when a single pair does not fit. */
int fxc_plan_xc_pairs(int64_t npairs, int64_t nwin, int32_t nchan, int64_t spec_pitch, const fxc_xc_shape *shape,
                      int method, int has_mask, int64_t budget_bytes, int64_t *pairs_per_call,
                      int64_t *bytes_per_call);
/* Device bytes of one stacking batch of ncf_pws (mode 0) / ncf_tfpws (mode 1):
 * the executables' trace, group, weight, linear and output buffers plus the
 * library scratch of fxc_pws_run / fxc_tfpws_run for the batch
 * (max_groups_per_pair: the largest substack-group count of one pair). */
int fxc_stack_batch_bytes(int mode, int64_t ntraces, int32_t npairs, int64_t ngroups, int64_t max_groups_per_pair,
                          int32_t nsamples, int64_t *bytes);
/* Largest batch (in traces, whole pairs of traces_per_pair) whose bytes fit
 * budget_bytes. Replaces select_tfpws_resident_chunk_plan
 * (native/tfpws/include/tfpws_schedule.hpp:149-217): this library forms
 * S-transform voices in shared memory, so its footprint depends on the pair
 * batch, not on a frequency chunk. FXC_ERR_NOMEM when one pair does not fit. */
int fxc_plan_stack_traces(int mode, int32_t nsamples, int32_t traces_per_pair, int32_t substack,
                          int64_t budget_bytes, int64_t *max_traces, int64_t *bytes_per_batch);

/* ---- SourcePack index over xcpack output (host only, no GPU) ------------------ */

typedef struct fxc_sourcepack_totals {
  int64_t timestamps, records, sources, bytes_indexed;
} fxc_sourcepack_totals;
typedef struct fxc_sourcepack_async fxc_sourcepack_async;

/* Per-timestamp SourcePack indexes of an xc output (the xcpack folder, or
 * the folder holding it): <out_dir>/<timestamp>/{sourcepack_index.tsv,
 * _SUCCESS}. Replaces build_sourcepack (timestamp NULL: every timestamp of
 * the TSVs, the workspace manifest and the .done markers; out_dir NULL:
 * <xcpack>/../sourcepack) and build_sourcepack_timestamp (timestamp set:
 * that timestamp from its own TSVs), fastxc/operators/sourcepack/
 * builder.py:163-271. sort_within_source orders rows by path id, component
 * slot, source key, receiver key, input order. progress_file (may be NULL)
 * receives the two-line progress sidecar. The resolved output folder is
 * written to out_path and the indexed timestamp folder names, one per line
 * in index order, to names (each when its capacity is > 0; truncated to
 * it). FXC_ERR_NOTFOUND for a missing folder or pack file, FXC_ERR_IO for a
 * malformed TSV. */
int fxc_sourcepack_build(const char *xc_root, const char *out_dir, const char *timestamp, int sort_within_source,
                         const char *progress_file, fxc_sourcepack_totals *out, char *out_path,
                         size_t out_path_cap, char *names, size_t names_cap);
/* Background indexing of each timestamp as soon as its .done marker
 * appears, polled every poll_interval_s (>= 0.5 s): replaces
 * AsyncSourcePackMaterializer (builder.py:27-159). finish stops the poller,
 * indexes what is left, writes the global _SUCCESS when mark_success (else
 * removes it and records status_message in the progress sidecar) and frees
 * the handle. */
int fxc_sourcepack_async_start(const char *xc_root, const char *out_dir, int sort_within_source,
                               const char *progress_file, double poll_interval_s, fxc_sourcepack_async **out);
int fxc_sourcepack_async_finish(fxc_sourcepack_async *a, int mark_success, const char *status_message,
                                fxc_sourcepack_totals *out);

/* Allocation-free variant of fxc_xc_run. No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc (a host framework that
 * owns all device memory through its own pool, or a job whose device
 * footprint is fixed at start-up). It allocates no device memory: its pair
 * tiles, FFT tables and stacked spectra live in one file-scope 64 MiB device
 * array that every GPU loading the library holds until exit. Takes the pair
 * list on the host (h_src, h_rec as in fxc_pairplan_create) and the same
 * device inputs/outputs as fxc_xc_run; FXC_XC_PLAIN method only.
 * Limits: nfft <= 40960 with nfft/2 a product of 2, 4, 8 and odd primes up
 * to 31 (the one-CTA transform), and tiles + tables + npairs *
 * round_up(nspec, 4) * 8 bytes within 64 MiB (about 450 pairs at nspec
 * 18523); else FXC_ERR_INVALID / FXC_ERR_UNSUPPORTED with the sizes in the
 * message. The pair tiles and FFT tables are built on the host inside the
 * call and copied into the array on the context's stream.
 * Set-up: the first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current and keeps it for the rest
 * of the process; make that first call before any stream capture begins.
 * A device reset (cudaDeviceReset) invalidates the kept address, so it is
 * not supported between calls. All calls share the array and it keeps the
 * last call's contents (each call rewrites everything it reads, nothing
 * needs clearing); calls whose work overlaps on the GPU race and must be
 * serialised by the caller. */
int fxc_xc_run_noalloc(fxc_ctx *ctx, const int32_t *h_src, const int32_t *h_rec, int64_t npairs,
                       const float *d_spec, int64_t nwin, int32_t nchan, int64_t spec_pitch,
                       const uint8_t *d_mask, float scale, const fxc_xc_shape *shape,
                       float *d_ncf);

#ifdef __cplusplus
}
#endif

#endif /* FASTXC_GB300_H */
