// Exact FP64-equivalent column sums of float32 traces in int64 fixed point
// (the cross-timestamp linear stack).
#pragma once

#include <cstdint>

namespace fxc {

// out[p, t] = float(sum_k double(tr[off_p + k, t]) / count_p), the sum in
// trace order (as _linear_stack_group accumulates: accum = first record in
// FP64, accum += each next record).
//
// GB300 runs FP64 adds at a small fraction of its FP32/INT32 rate, so the
// sequential FP64 sum (and the float -> double conversions) bound a direct
// restatement far below HBM speed. The sum is formed instead in int64
// fixed point, which is exact: the positive and the negative terms in two
// accumulators (their difference is the sum, their sum bounds every partial
// sum). When every partial sum s_k = x_0 + ... + x_k of the column is a
// double (a multiple of 2^L, L at or below the lowest set bit of every term,
// of magnitude below 2^(L+53)), each FP64 addition of the reference is exact
// too, so its result equals the exact sum bit for bit. A column for which the
// bound does not prove exactness (a term whose low bits fall below the
// accumulator's unit, a partial sum that may need more than 53 bits, a NaN or
// an infinity) is summed again by the FP64 loop itself. Signed zeros follow
// IEEE round-to-nearest: the sum is -0 only when every term is -0.
//
// Each thread owns V samples (T apart, coalesced), so V independent chains
// and loads are in flight per trace.

struct ExactCol {
  unsigned long long pos, neg;  // sums of the positive / negative terms' magnitudes, in units of 2^unit
  int unit;                     // exponent of one unit (the largest term exponent - G); kExactBad: no proof
  uint32_t lo_mag;              // magnitude bits of 2^(unit+23): the fast window starts here (0x80000000: none)
  uint32_t minmag;              // smallest nonzero magnitude (bits) among the terms; bit 31 cleared by a +0 term
};

constexpr int kExactBad = 1 << 24;  // a unit above every float exponent

// Terms keep at most 24 + G bits above the unit, G = min(31, 38 - bits(count)),
// so pos + neg <= count * 2^(24+G) < 2^62. A term whose magnitude bits lie in
// [lo_mag, lo_mag + ((G+1) << 23)) is a normal float with unit <= xe <=
// unit + G (|x| = m * 2^xe, m < 2^24): the fast path, one 32x32->64-bit
// multiply-add m * 2^(xe-unit) with no branch.
__device__ __forceinline__ void exact_init(ExactCol& c) {
  c.pos = 0;
  c.neg = 0;
  c.unit = -(1 << 20);  // below every float exponent: the first term sets it
  c.lo_mag = 0x80000000u;
  c.minmag = 0xffffffffu;
}

__device__ __forceinline__ int exact_count_bits(int cnt) { return min(31, 38 - (32 - __clz(cnt > 0 ? cnt : 1))); }

// Lower bound on the lowest set bit of a term with magnitude bits mag.
__device__ __forceinline__ int exact_low(uint32_t mag) { return (int)max(mag >> 23, 1u) - 150; }

__device__ __forceinline__ void exact_add_fast(ExactCol& c, uint32_t b, uint32_t diff) {
  const uint32_t m = (b & 0x7fffffu) | 0x800000u;
  c.minmag = min(c.minmag, b & 0x7fffffffu);
  const uint32_t pw = 1u << (diff >> 23);
  if (b >> 31)
    c.neg += (unsigned long long)m * pw;
  else
    c.pos += (unsigned long long)m * pw;
}

// Any term: zeros, subnormals, NaN and infinities (which enter with
// xe = 105, above every finite float: the unit ends at 105 - G and the
// column goes to the FP64 loop), terms above the window (the unit is raised,
// exact when every earlier term is a multiple of the new unit) and below it
// (exact only when the dropped bits are zero).
__device__ __forceinline__ void exact_add_any(ExactCol& c, uint32_t b, int G) {
  const uint32_t mag = b & 0x7fffffffu;
  if (mag == 0u) {
    if (b == 0u) c.minmag &= 0x7fffffffu;
    return;
  }
  const uint32_t e = mag >> 23;
  uint32_t m = e ? ((mag & 0x7fffffu) | 0x800000u) : mag;
  const int xe = (e ? (int)e : 1) - 150;
  c.minmag = min(c.minmag, mag);
  int sh = xe - c.unit;
  if (sh > G) {
    const int d = sh - G;
    if (exact_low(c.minmag) < c.unit + d) {
      c.unit = kExactBad;
      c.lo_mag = 0x80000000u;
      return;
    }
    c.pos = d >= 63 ? 0ull : (c.pos >> d);
    c.neg = d >= 63 ? 0ull : (c.neg >> d);
    c.unit += d;
    c.lo_mag = c.unit + 150 >= 1 ? (uint32_t)(c.unit + 150) << 23 : 0x80000000u;
    sh = G;
  } else if (sh < 0) {
    if (xe + (__ffs((int)m) - 1) < c.unit) {
      c.unit = kExactBad;
      c.lo_mag = 0x80000000u;
      return;
    }
    m >>= -sh;  // -sh <= trailing zeros of m <= 23
    sh = 0;
  }
  const unsigned long long v = (unsigned long long)m << sh;
  if (b >> 31)
    c.neg += v;
  else
    c.pos += v;
}

// The FP64 sum when exactness is proven; false otherwise.
__device__ __forceinline__ bool exact_result(const ExactCol& c, int G, double* s) {
  if (c.unit + G >= 105) return false;  // NaN, infinity or no proof
  // every s_k is a multiple of 2^low of magnitude <= (pos + neg) * 2^unit
  const unsigned long long sabs = c.pos + c.neg;
  const int room = exact_low(c.minmag) - c.unit + 53;
  if (room < 64 && (sabs >> room) != 0ull) return false;
  if (c.pos == c.neg) {
    // every nonzero term adds at least one unit to sabs; -0 only when every term is -0
    *s = (sabs != 0ull || c.minmag != 0xffffffffu) ? 0.0 : -0.0;
    return true;
  }
  // |pos - neg| < 2^53 in units of 2^(low-unit): the conversion is exact;
  // the unit lies in [-180, 104], a normal double exponent
  const long long acc = (long long)(c.pos - c.neg);
  *s = (double)acc * __hiloint2double((c.unit + 1023) << 20, 0);
  return true;
}

// The reference's own sequence of FP64 additions over one column; loads
// issued eight at a time.
__device__ __noinline__ double fp64_column_sum(const float* __restrict__ col, int64_t stride, int cnt) {
  double s = (double)__ldg(col);
  int k = 1;
  for (; k + 8 <= cnt; k += 8) {
    float x[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) x[j] = __ldg(col + (int64_t)(k + j) * stride);
#pragma unroll
    for (int j = 0; j < 8; ++j) s += (double)x[j];
  }
  for (; k < cnt; ++k) s += (double)__ldg(col + (int64_t)k * stride);
  return s;
}

// All cnt rows of the columns owned by this thread into col, through a
// register ring of NBUF rows: blocks of R rows are summed (one branch per
// block, taken when every term of the block is in its window) while the
// NBUF - R rows after them are in flight (the ring index of every row is a
// compile-time constant). FULL: every
// column of the CTA lies inside the trace, so all V loads share one address.
template <int T, int V, int NBUF, int R, bool FULL>
__device__ __forceinline__ void linear_stack_rows(ExactCol (&col)[V], const float* __restrict__ colp,
                                                  const int (&dv)[V], int64_t n, int cnt, int G) {
  static_assert(NBUF % R == 0, "the ring holds whole blocks");
  const uint32_t span = (uint32_t)(G + 1) << 23;
  auto load_row = [&](int k, float (&x)[V], bool guard) {
    const float* row = colp + (int64_t)k * n;
#pragma unroll
    for (int v = 0; v < V; ++v) {
      // rows past the count load as -0, which leaves every sum unchanged
      if (guard && k >= cnt)
        x[v] = -0.f;
      else
        x[v] = __ldg(row + (FULL ? v * T : dv[v]));
    }
  };
  float x[NBUF][V];
  auto add_block = [&](int j0) {
    uint32_t diff[R][V];
    bool fast = true;
#pragma unroll
    for (int r = 0; r < R; ++r)
#pragma unroll
      for (int v = 0; v < V; ++v) {
        diff[r][v] = (__float_as_uint(x[j0 + r][v]) & 0x7fffffffu) - col[v].lo_mag;
        fast = fast && diff[r][v] < span;
      }
    if (fast) {
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int v = 0; v < V; ++v) exact_add_fast(col[v], __float_as_uint(x[j0 + r][v]), diff[r][v]);
    } else {
      // in row order: a term may move the unit and the window of the next
#pragma unroll
      for (int r = 0; r < R; ++r)
#pragma unroll
        for (int v = 0; v < V; ++v) exact_add_any(col[v], __float_as_uint(x[j0 + r][v]), G);
    }
  };
  // slot s holds rows s, s + NBUF, ...; before block j is summed, the slots
  // of the block before it are refilled with the rows NBUF - R ahead
#pragma unroll
  for (int j = 0; j < NBUF - R; ++j) load_row(j, x[j], true);
  int k = 0;
  // every row loaded in this loop (up to k + 2*NBUF - R - 1) is below the count
  for (; k + 2 * NBUF - R <= cnt; k += NBUF) {
#pragma unroll
    for (int j = 0; j < NBUF; j += R) {
#pragma unroll
      for (int r = 0; r < R; ++r) load_row(k + j + NBUF - R + r, x[(j + NBUF - R + r) % NBUF], false);
      add_block(j);
    }
  }
  for (; k < cnt; k += NBUF) {
#pragma unroll
    for (int j = 0; j < NBUF; j += R) {
#pragma unroll
      for (int r = 0; r < R; ++r) load_row(k + j + NBUF - R + r, x[(j + NBUF - R + r) % NBUF], true);
      add_block(j);
    }
  }
}

// One CTA of T threads sums T*V consecutive samples (T apart per thread) of
// pair blockIdx.y.
template <int T, int V, int NBUF, int R>
__device__ __forceinline__ void linear_stack_cta(const float* __restrict__ traces,
                                                 const int64_t* __restrict__ offs,
                                                 const int32_t* __restrict__ counts, int n,
                                                 float* __restrict__ out) {
  const int p = blockIdx.y;
  const int64_t off = offs[p];
  const int cnt = counts[p];
  const int t0 = blockIdx.x * (T * V) + threadIdx.x;
  const int G = exact_count_bits(cnt);
  const float* base = traces + off * n;
  ExactCol col[V];
#pragma unroll
  for (int v = 0; v < V; ++v) exact_init(col[v]);
  // columns past the trace end read the last sample (results dropped)
  const int tc = min(t0, n - 1);
  int dv[V];
#pragma unroll
  for (int v = 0; v < V; ++v) dv[v] = min(t0 + v * T, n - 1) - tc;
  if (cnt > 0) {
    if ((int)(blockIdx.x + 1) * (T * V) <= n)
      linear_stack_rows<T, V, NBUF, R, true>(col, base + tc, dv, n, cnt, G);
    else
      linear_stack_rows<T, V, NBUF, R, false>(col, base + tc, dv, n, cnt, G);
  }
#pragma unroll
  for (int v = 0; v < V; ++v) {
    const int t = t0 + v * T;
    if (t >= n) continue;
    double s;
    if (cnt > 0 && !exact_result(col[v], G, &s)) s = fp64_column_sum(base + t, n, cnt);
    out[(int64_t)p * n + t] = cnt > 0 ? (float)(s / (double)cnt) : 0.f;
  }
}

}  // namespace fxc
