// Kernel (b), lattice part: batched k <-> r FFTs over 1-3 periodic mesh
// dimensions, for every frequency slice and target element.
//
// Restates c++/triqs_tprf/fourier/fourier_lattice.cpp:28-59 with
// fourier_common.cpp:26-53: a multi-dimensional DFT over the mesh dims with
// the target elements as the batch (FFTW howmany = n_target, stride =
// n_target). k -> r is FFTW_FORWARD divided by N_k; r -> k is FFTW_BACKWARD,
// unscaled. lattice/fourier.hpp:166-231 loops over the frequency slices.
//
// Design: the array is viewed as [outer, n, inner] for each transformed axis
// (target index fastest, as in HBM). One CTA loads a tile of up to 64
// consecutive columns of the flattened (outer, inner) index into shared
// memory with coalesced row reads (in digit-reversed row order), runs an
// in-place mixed-radix FFT on all columns at once and writes the tile back. One pass per mesh
// dimension with n > 1; later passes run in place. The butterflies run in
// double-float pairs on the FP32 pipe by default (tprf_set_arithmetic).
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <type_traits>

#include "common.cuh"
#include "tma.cuh"

#include <cudaTypedefs.h>

namespace tprf {
namespace {

constexpr int kLoadBatch = 8;  // tile loads per thread issued together

// Leading part of a pass to leave out when the bubble's input was real
// (gmax, see gmax_says_real): the negative bosonic frequencies, which the
// last pass stores from their partner rows (RowMirror). `columns` counts the
// pass's own units (the axis pass: flattened columns; the plane pass: outer
// indices); 0 = none.
struct SkipRows {
  const unsigned *gmax;
  long columns;
};

// The negative frequencies written by the last pass of a lattice transform.
// On a real bubble the rows satisfy x(-w, q) = conj(x(w, -q)) exactly, so the
// pass that finishes row j (counted from the pass's base pointer; its partner
// is row c - j) also stores the conjugate at the partner row and the negated k
// point. Rows with c - j > j belong to their partner and are not stored; the
// row with c - j == j (w = 0) has none. The conjugate is the stored value with
// the sign bits of its imaginary words flipped, so the pair is exact bit for
// bit. e1, e2: the mesh dims after the transformed axis (1 where absent); the
// dims before it are trivial, as the last pass transforms the slowest
// non-trivial axis.
struct RowMirror {
  const unsigned *gmax;  // words of the real-input test (gmax_says_real); null: unconditional
  long c;
  int e1, e2;
  int on;
  __device__ __forceinline__ bool active() const { return on && (gmax == nullptr || gmax_says_real(gmax)); }
};
constexpr RowMirror kNoRowMirror{nullptr, 0, 1, 1, 0};
constexpr long kNoPartner = -0x7fffffffffffffffL - 1;  // a column without a partner store


template <class E> __device__ __forceinline__ E load_el(double2 z);
template <> __device__ __forceinline__ double2 load_el<double2>(double2 z) { return z; }
template <> __device__ __forceinline__ cdf load_el<cdf>(double2 z) { return to_cdf(z); }
__device__ __forceinline__ double2 store_el(double2 z, double s, dfl, bool scaled) { return scaled ? cscale(z, s) : z; }
__device__ __forceinline__ double2 store_el(cdf z, double, dfl sd, bool scaled) {
  // one FP64 addition per part (to_double_add): the lattice passes leave the FP64
  // pipe nearly idle, and this takes fewer instructions than the bit-operation form
  const cdf w = scaled ? cscale(z, sd) : z;
  return make_double2(to_double_add(w.x), to_double_add(w.y));
}

// Element i of a pass's input or output in either storage format: complex128,
// or (DF) double-float pairs (re.hi, re.lo, im.hi, im.lo), the same 16 bytes.
// Passes of one transform hand each other double-float pairs, so only the
// transform's own input and output are converted.
template <class E, bool DF>
__device__ __forceinline__ E load_in(const void *p, long i) {
  if constexpr (DF) {
    static_assert(std::is_same<E, cdf>::value, "double-float storage needs double-float arithmetic");
    return reinterpret_cast<const cdf *>(p)[i];
  } else {
    return load_el<E>(reinterpret_cast<const double2 *>(p)[i]);
  }
}
// The same in two steps, so that a batch of loads can be in flight before any
// is converted: the raw 16 bytes, then the element.
template <bool DF> struct RawOf { using type = double2; };
template <> struct RawOf<true> { using type = cdf; };
template <class E, bool DF>
__device__ __forceinline__ typename RawOf<DF>::type load_raw(const void *p, long i) {
  return reinterpret_cast<const typename RawOf<DF>::type *>(p)[i];
}
template <class E> __device__ __forceinline__ E from_raw(double2 z) { return load_el<E>(z); }
template <class E> __device__ __forceinline__ E from_raw(cdf z) { return z; }
template <class E> __device__ __forceinline__ E zero_el();
template <> __device__ __forceinline__ double2 zero_el<double2>() { return make_double2(0.0, 0.0); }
template <> __device__ __forceinline__ cdf zero_el<cdf>() { return cdf{dfl{0.f, 0.f}, dfl{0.f, 0.f}}; }
template <class E, bool DF>
__device__ __forceinline__ void store_out(void *p, long i, E z, double s, dfl sd, bool scaled) {
  if constexpr (DF) {
    reinterpret_cast<cdf *>(p)[i] = scaled ? cscale(z, sd) : cnorm(z);
  } else {
    reinterpret_cast<double2 *>(p)[i] = store_el(z, s, sd, scaled);
  }
}

// The 16 bytes a pass stores for element z, and the same with the imaginary
// part's sign bits flipped: complex128 {x, y} has the sign of y in bit 31 of
// .w; double-float {x.hi, x.lo, y.hi, y.lo} has those of y.hi and y.lo in .z
// and .w (a negation would run on the FP64 pipe).
union Bits16 {
  int4 i;
  double2 d;
  cdf f;
};
template <class E, bool DF>
__device__ __forceinline__ int4 stored_bits(E z, double s, dfl sd, bool scaled) {
  Bits16 b;
  if constexpr (DF)
    b.f = scaled ? cscale(z, sd) : cnorm(z);
  else
    b.d = store_el(z, s, sd, scaled);
  return b.i;
}
template <bool DF>
__device__ __forceinline__ int4 conj_bits(int4 v) {
  if constexpr (DF) v.z ^= (int)0x80000000u;
  v.w ^= (int)0x80000000u;
  return v;
}

// A pass on the compact canonical orbital columns of a real bubble
// (CompactChi), active when gmax is set and the words say canon_says_yes. The
// plane pass then runs in place on buf ([outer][n1][n2][n_target], n_target =
// nc); the last (axis) pass reads buf ([outer][n][inner], inner = e1 e2 nc,
// outer = the rows w >= 0) and stores, for the element (w, i, k, j) of the
// canonical column t = ocan[j] and its reflection tr = orev[j]:
//   (w, i, k, t) and, unless t is a palindrome, (w, -i, -k, tr) (the same value:
//   chi0(w, -q)_dcba = chi0(w, q)_abcd), and for w > 0 the conjugates at
//   (-w, -i, -k, t) and (-w, i, k, tr): every column of both signs of w in out.
struct CompactPass {
  const unsigned *gmax;  // null: off
  void *buf;
  long outer, n_target;  // plane: rows x (dims before the plane), nc; axis: rows, e1 e2 nc
  int nc, nb4;
  // axis: compact row o (frequency w0 + o) goes to output row row0 + o, its
  // conjugate partner (for w0 + o > 0) to row prow0 - o
  long row0, prow0, w0;
  const int *ocan, *orev;
  // axis: the k points in tile order (get_k_pair_order), so that the columns of
  // k and -k, which fill each other's output rows, are stored close in time and
  // their 32-byte sectors reach DRAM whole
  const int *kperm;
  __device__ __forceinline__ bool active() const { return gmax != nullptr && canon_says_yes(gmax); }
};
constexpr CompactPass kNoCompact{nullptr, nullptr, 0, 0, 0, 0, 0, 0, 0, nullptr, nullptr, nullptr};

template <bool FWD, class E, bool IN_DF, bool OUT_DF>
__global__ void __launch_bounds__(256) lattice_axis_kernel(const void *in, void *out, long ncols_total,
                                                           long inner, int ncol, int lgcol, FftDesc d, double scale,
                                                           SkipRows skip, RowMirror mir, CompactPass cp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int n = d.n;
  E *a = reinterpret_cast<E *>(smem_raw);
  E *b = d.has_generic ? a + (size_t)n * ncol : nullptr;
  long *base = reinterpret_cast<long *>(smem_raw + (size_t)(d.has_generic ? 2 : 1) * n * ncol * sizeof(E));
  long *pbase = base + ncol;  // partner stores (the launcher sizes shared memory for them when mir.on)
  long *cdst = base + ncol;   // compact pass: four store bases per column, [4][ncol]
  // The tile is ncol consecutive columns of the flattened (outer, inner) index;
  // element (row, column f) sits at (f / inner) * n * inner + row * inner + f % inner.
  const long f0 = blockIdx.x * (long)ncol;
  const bool cm = cp.active();
  const void *src = cm ? cp.buf : in;
  const long istride = cm ? cp.n_target : inner;  // row stride of the input
  if (cm) {
    if (f0 >= cp.outer * cp.n_target) return;  // the grid is sized for the full layout
  } else if (f0 + ncol <= skip.columns && gmax_says_real(skip.gmax)) {
    return;  // rows the partner rows fill
  }
  const bool mirror = !cm && mir.active();
  for (int c = threadIdx.x; c < ncol; c += blockDim.x) {
    const long f = f0 + c;
    if (cm) {
      long bs = -1, s[4] = {kNoPartner, kNoPartner, kNoPartner, kNoPartner};
      if (f < cp.outer * cp.n_target) {
        const long o = f / cp.n_target, rem = f - o * cp.n_target;
        const long pos = rem / cp.nc;
        const int j = (int)(rem - pos * cp.nc);
        const long kk = cp.kperm[pos];
        const long k1 = kk / mir.e2, k2 = kk - k1 * mir.e2;
        const long mk = (k1 ? mir.e1 - k1 : 0) * (long)mir.e2 + (k2 ? mir.e2 - k2 : 0);
        const int t = cp.ocan[j], tr = cp.orev[j];
        const long O = cp.row0 + o, P = cp.prow0 - o;
        bs = o * n * cp.n_target + kk * cp.nc + j;
        s[0] = O * n * inner + kk * cp.nb4 + t;
        if (tr != t) s[1] = O * n * inner + mk * cp.nb4 + tr;
        if (cp.w0 + o > 0) {
          s[2] = P * n * inner + mk * cp.nb4 + t;
          if (tr != t) s[3] = P * n * inner + kk * cp.nb4 + tr;
        }
      }
      base[c] = bs;
      for (int q = 0; q < 4; ++q) cdst[q * ncol + c] = s[q];
      continue;
    }
    const long o = f / inner;
    long bs = (f < ncols_total) ? o * n * inner + (f - o * inner) : -1;
    if (mirror) {
      // outer index o is the row (the dims before the axis are trivial); the
      // partner element of (row i, inner (k1, k2, t)) is (c - o, -i, -k1, -k2, t)
      long pb = kNoPartner;
      const long prow = mir.c - o;
      if (bs >= 0 && prow > o) bs = -1;  // stored by the partner row's tile
      if (bs >= 0 && prow < o) {
        const long n_target = inner / ((long)mir.e1 * mir.e2);
        const long rem = f - o * inner, kk = rem / n_target, t = rem - kk * n_target;
        const long k1 = kk / mir.e2, k2 = kk - k1 * mir.e2;
        const long mk = (k1 ? mir.e1 - k1 : 0) * (long)mir.e2 + (k2 ? mir.e2 - k2 : 0);
        pb = prow * n * inner + mk * n_target + t;
      }
      pbase[c] = pb;
    }
    base[c] = bs;
  }
  __syncthreads();
  const int tile = n * ncol;
  // kLoadBatch loads per thread in flight before the first is converted and stored
  for (int w0 = threadIdx.x; w0 < tile; w0 += kLoadBatch * blockDim.x) {
    typename RawOf<IN_DF>::type v[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int w = w0 + u * blockDim.x;
      const int c = w & (ncol - 1), row = w >> lgcol;
      const long bs = w < tile ? base[c] : -1;
      if (bs >= 0) v[u] = load_raw<E, IN_DF>(src, bs + (long)row * istride);
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int w = w0 + u * blockDim.x;
      if (w >= tile) break;
      const int c = w & (ncol - 1), row = w >> lgcol;
      a[d.rev[row] * ncol + c] = base[c] >= 0 ? from_raw<E>(v[u]) : zero_el<E>();
    }
  }
  E *r = fft_smem<FWD>(a, b, d, ncol);
  const bool scaled = scale != 1.0;
  const dfl sd = split_double(scale);
  if (cm) {
    int4 *o4 = reinterpret_cast<int4 *>(out);
    for (int w = threadIdx.x; w < tile; w += blockDim.x) {
      const int c = w & (ncol - 1), row = w >> lgcol;
      if (base[c] < 0) continue;
      const long nrow = row ? n - row : 0;
      const int4 v = stored_bits<E, OUT_DF>(r[row * ncol + c], scale, sd, scaled);
      o4[cdst[c] + (long)row * inner] = v;
      const long s1 = cdst[ncol + c], s2 = cdst[2 * ncol + c], s3 = cdst[3 * ncol + c];
      if (s1 != kNoPartner) o4[s1 + nrow * inner] = v;
      if (s2 != kNoPartner) o4[s2 + nrow * inner] = conj_bits<OUT_DF>(v);
      if (s3 != kNoPartner) o4[s3 + (long)row * inner] = conj_bits<OUT_DF>(v);
    }
    return;
  }
  if (mirror) {
    int4 *o4 = reinterpret_cast<int4 *>(out);
    for (int w = threadIdx.x; w < tile; w += blockDim.x) {
      const int c = w & (ncol - 1), row = w >> lgcol;
      const long bs = base[c];
      if (bs < 0) continue;
      const int4 v = stored_bits<E, OUT_DF>(r[row * ncol + c], scale, sd, scaled);
      o4[bs + (long)row * inner] = v;
      const long pb = pbase[c];
      if (pb != kNoPartner) o4[pb + (long)(row ? n - row : 0) * inner] = conj_bits<OUT_DF>(v);
    }
    return;
  }
  for (int w = threadIdx.x; w < tile; w += blockDim.x) {
    const int c = w & (ncol - 1), row = w >> lgcol;
    const long bs = base[c];
    if (bs >= 0) store_out<E, OUT_DF>(out, bs + (long)row * inner, r[row * ncol + c], scale, sd, scaled);
  }
}

template <bool FWD, class E, bool IN_DF, bool OUT_DF>
int launch_axis_as(const void *in, void *out, long outer, int n, long inner, double scale, cudaStream_t stream,
                   SkipRows skip = SkipRows{nullptr, 0}, RowMirror mir = kNoRowMirror, CompactPass cp = kNoCompact) {
  FftDesc d;
  int st = get_fft(n, &d);
  if (st) return st;
  // Tile of up to 64 columns (a power of two dividing the 256 threads), limited
  // by shared memory: one buffer of n x ncol elements (two with a generic radix)
  // and the column offsets (twice with partner stores, five for a compact pass).
  const int bufs = d.has_generic ? 2 : 1;
  const size_t offs = (cp.gmax ? 5 : mir.on ? 2 : 1) * sizeof(long);
  const size_t budget = (size_t)std::min(max_smem_optin(), 200 * 1024);
  int ncol = 64;
  while (ncol > 1 && (size_t)bufs * n * ncol * sizeof(E) + ncol * offs > budget) ncol /= 2;
  const long ncols_total = outer * inner;
  while (ncol > 8 && ncol / 2 >= ncols_total) ncol /= 2;
  const size_t smem = (size_t)bufs * n * ncol * sizeof(E) + ncol * offs;
  if (smem > budget) return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "lattice FFT: mesh dimension too long for one CTA");
  int lg = 0;
  while ((1 << lg) < ncol) ++lg;
  const long blocks = (ncols_total + ncol - 1) / ncol;
  if (blocks > 0x7fffffffL) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: too many tiles");
  auto kern = lattice_axis_kernel<FWD, E, IN_DF, OUT_DF>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)blocks, 256, smem, stream>>>(in, out, ncols_total, inner, ncol, lg, d, scale, skip, mir, cp);
  TPRF_KERNEL_LAUNCHED("lattice_axis_kernel");
  return TPRF_OK;
}

// Storage formats of a pass: complex128 (0) or double-float pairs (1) for its
// input and output; double-float only with double-float arithmetic.
template <bool FWD>
int launch_axis(const void *in, bool in_df, void *out, bool out_df, long outer, int n, long inner, double scale,
                cudaStream_t stream, SkipRows skip = SkipRows{nullptr, 0}, RowMirror mir = kNoRowMirror,
                CompactPass cp = kNoCompact) {
  if (arith_mode() == kArithFP64) {
    if (in_df || out_df) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: double-float storage in FP64 mode");
    return launch_axis_as<FWD, double2, false, false>(in, out, outer, n, inner, scale, stream, skip, mir, cp);
  }
  if (in_df && out_df)
    return launch_axis_as<FWD, cdf, true, true>(in, out, outer, n, inner, scale, stream, skip, mir, cp);
  if (in_df) return launch_axis_as<FWD, cdf, true, false>(in, out, outer, n, inner, scale, stream, skip, mir, cp);
  if (out_df) return launch_axis_as<FWD, cdf, false, true>(in, out, outer, n, inner, scale, stream, skip, mir, cp);
  return launch_axis_as<FWD, cdf, false, false>(in, out, outer, n, inner, scale, stream, skip, mir, cp);
}

// Two adjacent mesh axes in one pass: the array is [outer, n1, n2, n_target]
// and a CTA transforms the n1 x n2 plane of nt consecutive targets. The tile
// sits in shared memory as [i1][i2][t] with both axes digit-reversed; the
// n2-point transforms see columns (i1, t) with element stride nt, the
// n1-point ones columns (i2, t) with stride n2 * nt. Each element is read,
// converted, written and converted back once for both axes. n1, n2 and nt are
// powers of two with n1 * nt and n2 * nt dividing the 256 threads.
template <bool FWD, class E, bool IN_DF, bool OUT_DF>
__global__ void __launch_bounds__(256) lattice_plane_kernel(const void *in, void *out, long outer, long n_target,
                                                            int nt, int lgt, FftDesc d1, FftDesc d2, int lg2,
                                                            double scale, SkipRows skip, RowMirror mir,
                                                            CompactPass cp) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  E *a = reinterpret_cast<E *>(smem_raw);
  const int n1 = d1.n, n2 = d2.n, P = n1 * n2;
  // a compact pass runs in place on the canonical orbital columns (the grid is
  // sized for the full layout; the CTAs past the compact tiles leave)
  const bool cm = cp.active();
  if (cm) {
    in = cp.buf;
    out = cp.buf;
    outer = cp.outer;
    n_target = cp.n_target;
  }
  const long tiles_t = (n_target + nt - 1) / nt;
  const long o = blockIdx.x / tiles_t;
  if (o >= outer) return;
  if (!cm && o < skip.columns && gmax_says_real(skip.gmax)) return;  // rows the partner rows fill
  // partner stores: o is the row (the dims before the plane are trivial)
  const bool mirror = !cm && mir.active();
  const long prow = mir.c - o;
  if (mirror && prow > o) return;  // stored by the partner row's tiles
  const long t0 = (blockIdx.x - o * tiles_t) * (long)nt;
  const int ntv = (int)min((long)nt, n_target - t0);
  const long gbase = o * P * n_target + t0;
  for (int w0 = threadIdx.x; w0 < P * nt; w0 += kLoadBatch * blockDim.x) {
    typename RawOf<IN_DF>::type v[kLoadBatch];
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int w = w0 + u * blockDim.x;
      const int t = w & (nt - 1), p = w >> lgt;
      if (w < P * nt && t < ntv) v[u] = load_raw<E, IN_DF>(in, gbase + (long)p * n_target + t);
    }
#pragma unroll
    for (int u = 0; u < kLoadBatch; ++u) {
      const int w = w0 + u * blockDim.x;
      if (w >= P * nt) break;
      const int t = w & (nt - 1), p = w >> lgt;
      const int i1 = p >> lg2, i2 = p & (n2 - 1);
      a[((d1.rev[i1] << lg2) + d2.rev[i2]) * nt + t] = t < ntv ? from_raw<E>(v[u]) : zero_el<E>();
    }
  }
  // axis 2: columns (i1, t), element i2 at i1 * n2 * nt + i2 * nt + t
  fft_smem<FWD>(a, (E *)nullptr, d2, n1 * nt, -1, ColLayout{nt, n2 * nt, lgt});
  // axis 1: columns (i2, t), element i1 at i1 * n2 * nt + (i2 * nt + t)
  E *r = fft_smem<FWD>(a, (E *)nullptr, d1, n2 * nt);
  const bool scaled = scale != 1.0;
  const dfl sd = split_double(scale);
  if (mirror) {
    // element (i1, i2, t) of row o, and its conjugate at (prow, -i1, -i2, t) for w != 0
    int4 *o4 = reinterpret_cast<int4 *>(out);
    const long pbase = prow * P * n_target + t0;
    for (int w = threadIdx.x; w < P * nt; w += blockDim.x) {
      const int t = w & (nt - 1), p = w >> lgt;
      if (t >= ntv) continue;
      const int4 v = stored_bits<E, OUT_DF>(r[p * nt + t], scale, sd, scaled);
      o4[gbase + (long)p * n_target + t] = v;
      if (prow < o) {
        const int i1 = p >> lg2, i2 = p & (n2 - 1);
        const int pm = (((n1 - i1) & (n1 - 1)) << lg2) | ((n2 - i2) & (n2 - 1));
        o4[pbase + (long)pm * n_target + t] = conj_bits<OUT_DF>(v);
      }
    }
    return;
  }
  for (int w = threadIdx.x; w < P * nt; w += blockDim.x) {
    const int t = w & (nt - 1), p = w >> lgt;
    if (t < ntv) store_out<E, OUT_DF>(out, gbase + (long)p * n_target + t, r[p * nt + t], scale, sd, scaled);
  }
}

// TMA-staged form of the plane pass (double-float arithmetic): persistent CTAs
// with two tile buffers. While the transforms of one tile run, the TMA unit
// copies the CTA's next tile into the other buffer (one 4-D box per tile,
// [i1][i2][t] in natural order as the box lays it out), so the tile loads no
// longer wait on DRAM latency. The transforms run decimation-in-frequency on
// the natural-order tile and the store reads the digit-reversed positions.
// Double-float input lands as it is; complex128 input is converted in place.

template <bool FWD, bool IN_DF, bool OUT_DF>
__global__ void __launch_bounds__(256) lattice_plane_tma_kernel(const __grid_constant__ CUtensorMap map, void *out,
                                                                long outer, long n_target, int nt, int lgt, FftDesc d1,
                                                                FftDesc d2, int lg2, double scale, unsigned *status,
                                                                unsigned long long wait_ns) {
  using E = cdf;
  extern __shared__ __align__(128) unsigned char smem_raw[];
  const int n1 = d1.n, n2 = d2.n, P = n1 * n2, tile_elems = P * nt;
  E *buf0 = reinterpret_cast<E *>(smem_raw);
  E *buf1 = buf0 + tile_elems;
  uint64_t *bar = reinterpret_cast<uint64_t *>(buf1 + tile_elems);
  const long tiles_t = (n_target + nt - 1) / nt;
  const long n_tiles = outer * tiles_t;
  const uint32_t tile_bytes = (uint32_t)tile_elems * 16u;
  auto issue = [&](long tile, int b) {
    const long o = tile / tiles_t;
    const int t0 = (int)((tile - o * tiles_t) * nt);
    mbar_arrive_expect_tx(&bar[b], tile_bytes);
    tma_load_4d(b ? buf1 : buf0, &map, 2 * t0, 0, 0, (int)o, &bar[b]);
  };
  if (threadIdx.x == 0) {
    mbar_init(&bar[0], 1);
    mbar_init(&bar[1], 1);
    fence_mbar_init();
    fence_async_shared();
    if ((long)blockIdx.x < n_tiles) issue(blockIdx.x, 0);
  }
  __syncthreads();
  const bool scaled = scale != 1.0;
  const dfl sd = split_double(scale);
  int k = 0;
  for (long tile = blockIdx.x; tile < n_tiles; tile += gridDim.x, ++k) {
    const int b = k & 1;
    const long nxt = tile + gridDim.x;
    if (threadIdx.x == 0 && nxt < n_tiles) {
      fence_async_shared();  // this CTA's earlier accesses to that buffer precede the copy
      issue(nxt, b ^ 1);
    }
    const bool ok = mbar_wait_timed(&bar[b], (uint32_t)((k >> 1) & 1), wait_ns);
    if (__syncthreads_or(!ok)) {
      // the wait ran out: record it, then let both copies this block has in
      // flight (this tile's and the next one's) land before leaving, each for at
      // most kTmaDrainNs, since they write this block's shared memory
      if (threadIdx.x == 0) {
        atomicOr(status, kDevErrTimeout);
        mbar_wait_timed(&bar[b], (uint32_t)((k >> 1) & 1), kTmaDrainNs);
        if (nxt < n_tiles) mbar_wait_timed(&bar[b ^ 1], (uint32_t)(((k + 1) >> 1) & 1), kTmaDrainNs);
      }
      __syncthreads();
      return;
    }
    E *a = b ? buf1 : buf0;
    if constexpr (!IN_DF) {
      for (int w = threadIdx.x; w < tile_elems; w += blockDim.x) a[w] = to_cdf(reinterpret_cast<const double2 *>(a)[w]);
    }
    // axis 2: columns (i1, t), element i2 at i1 * n2 * nt + i2 * nt + t
    fft_smem_dif<FWD>(a, d2, n1 * nt, ColLayout{nt, n2 * nt, lgt});
    // axis 1: columns (i2, t), element i1 at i1 * n2 * nt + (i2 * nt + t)
    fft_smem_dif<FWD>(a, d1, n2 * nt);
    const long o = tile / tiles_t;
    const long t0 = (tile - o * tiles_t) * (long)nt;
    const int ntv = (int)min((long)nt, n_target - t0);
    const long gbase = o * P * n_target + t0;
    for (int w = threadIdx.x; w < tile_elems; w += blockDim.x) {
      const int t = w & (nt - 1), p = w >> lgt;
      const int i1 = p >> lg2, i2 = p & (n2 - 1);
      if (t < ntv)
        store_out<E, OUT_DF>(out, gbase + (long)p * n_target + t, a[((d1.rev[i1] << lg2) + d2.rev[i2]) * nt + t],
                             scale, sd, scaled);
    }
    __syncthreads();  // the buffer is free for the tile after next
  }
}

bool pow2(int n) { return n > 0 && (n & (n - 1)) == 0; }
int log2i(int n) {
  int l = 0;
  while ((1 << l) < n) ++l;
  return l;
}

// Whether the plane pass serves axes of lengths n1, n2 (and with how many targets per tile).
int plane_targets(int n1, int n2, long n_target) {
  if (!pow2(n1) || !pow2(n2) || n1 < 2 || n2 < 2) return 0;
  const int big = std::max(n1, n2);
  if (big > 256) return 0;
  int nt = 256 / big;
  // shared memory: a plane of nt targets, at most 64 KB so that three CTAs share an SM
  while (nt > 1 && (size_t)n1 * n2 * nt * sizeof(double2) > 64 * 1024) nt /= 2;
  if ((size_t)n1 * n2 * nt * sizeof(double2) > 64 * 1024) return 0;
  // generic-radix stages need a second buffer: not used for powers of two
  while (nt > 1 && nt / 2 >= n_target) nt /= 2;
  return nt;
}

template <bool FWD, class E, bool IN_DF, bool OUT_DF>
int launch_plane_as(const void *in, void *out, long outer, int n1, int n2, long n_target, double scale,
                    cudaStream_t stream, SkipRows skip, RowMirror mir, CompactPass cp) {
  FftDesc d1, d2;
  int st = get_fft(n1, &d1);
  if (st) return st;
  if ((st = get_fft(n2, &d2))) return st;
  const int nt = plane_targets(n1, n2, n_target);
  if (nt < 1) return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "lattice FFT: plane pass does not apply");
  const size_t smem = (size_t)n1 * n2 * nt * sizeof(E);
  const long tiles = outer * ((n_target + nt - 1) / nt);
  if (tiles > 0x7fffffffL) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: too many tiles");
  auto kern = lattice_plane_kernel<FWD, E, IN_DF, OUT_DF>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)tiles, 256, smem, stream>>>(in, out, outer, n_target, nt, log2i(nt), d1, d2, log2i(n2), scale,
                                               skip, mir, cp);
  TPRF_KERNEL_LAUNCHED("lattice_plane_kernel");
  return TPRF_OK;
}

template <bool FWD>
int launch_plane(const void *in, bool in_df, void *out, bool out_df, long outer, int n1, int n2, long n_target,
                 double scale, cudaStream_t stream, SkipRows skip = SkipRows{nullptr, 0},
                 RowMirror mir = kNoRowMirror, CompactPass cp = kNoCompact) {
  if (arith_mode() == kArithFP64) {
    if (in_df || out_df) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: double-float storage in FP64 mode");
    return launch_plane_as<FWD, double2, false, false>(in, out, outer, n1, n2, n_target, scale, stream, skip, mir,
                                                       cp);
  }
  if (in_df && out_df)
    return launch_plane_as<FWD, cdf, true, true>(in, out, outer, n1, n2, n_target, scale, stream, skip, mir, cp);
  if (in_df)
    return launch_plane_as<FWD, cdf, true, false>(in, out, outer, n1, n2, n_target, scale, stream, skip, mir, cp);
  if (out_df)
    return launch_plane_as<FWD, cdf, false, true>(in, out, outer, n1, n2, n_target, scale, stream, skip, mir, cp);
  return launch_plane_as<FWD, cdf, false, false>(in, out, outer, n1, n2, n_target, scale, stream, skip, mir, cp);
}

// The TMA-staged plane pass with nt targets per tile (two tiles per CTA).
constexpr int kNotApplicable = 1;

template <bool FWD>
int launch_plane_tma_nt(const void *in, bool in_df, void *out, bool out_df, long outer, int n1, int n2,
                        long n_target, double scale, cudaStream_t stream, int nt) {
  const int P = n1 * n2;
  FftDesc d1, d2;
  int st = get_fft(n1, &d1);
  if (st) return st;
  if ((st = get_fft(n2, &d2))) return st;
  unsigned *status = device_status_word();
  if (!status) return TPRF_ERR_CUDA;
  // the array as FP64 words: [outer][n1][n2][n_target][2]
  const uint64_t dims[4] = {2 * (uint64_t)n_target, (uint64_t)n2, (uint64_t)n1, (uint64_t)outer};
  const uint64_t strides[3] = {16 * (uint64_t)n_target, 16 * (uint64_t)n_target * n2,
                               16 * (uint64_t)n_target * n2 * n1};
  const uint32_t box[4] = {2 * (uint32_t)nt, (uint32_t)n2, (uint32_t)n1, 1};
  CUtensorMap map;
  if ((st = encode_tensor_map_f64(&map, in, 4, dims, strides, box))) return st;
  const size_t smem = 2 * (size_t)P * nt * 16 + 16;
  const long tiles = outer * ((n_target + nt - 1) / nt);
  void (*kern)(const CUtensorMap, void *, long, long, int, int, FftDesc, FftDesc, int, double, unsigned *,
               unsigned long long);
  if (in_df)
    kern = out_df ? lattice_plane_tma_kernel<FWD, true, true> : lattice_plane_tma_kernel<FWD, true, false>;
  else
    kern = out_df ? lattice_plane_tma_kernel<FWD, false, true> : lattice_plane_tma_kernel<FWD, false, false>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  int per_sm = 0;
  TPRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
  const long grid = std::max(1L, std::min(tiles, (long)num_sms() * std::max(1, per_sm)));
  kern<<<(unsigned)grid, 256, smem, stream>>>(map, out, outer, n_target, nt, log2i(nt), d1, d2, log2i(n2), scale,
                                              status, device_wait_limit_ns());
  TPRF_KERNEL_LAUNCHED("lattice_plane_tma_kernel");
  return TPRF_OK;
}

// The plane pass: the TMA-staged form with the tile size the wisdom names
// (autotuner: measure mode on an out-of-place call, or tprf_autotune_load),
// else the plain form (kNotApplicable tells the caller to run it).
template <bool FWD>
int launch_plane_tma(const void *in, bool in_df, void *out, bool out_df, long outer, int n1, int n2, long n_target,
                     double scale, cudaStream_t stream) {
  if (arith_mode() == kArithFP64 || (reinterpret_cast<uintptr_t>(in) & 15) || outer > 0x7fffffffL ||
      2 * n_target > 0x7fffffffL || plane_targets(n1, n2, n_target) < 1)
    return kNotApplicable;
  const int P = n1 * n2;
  auto fits = [&](int nt) {
    return n1 * nt <= 256 && n2 * nt <= 256 && 256 % (n1 * nt) == 0 && 256 % (n2 * nt) == 0 &&
           ((size_t)P * nt * 16) % 128 == 0 && 2 * (size_t)P * nt * 16 + 16 <= (size_t)max_smem_optin() &&
           (nt == 1 || nt / 2 < n_target);
  };
  std::vector<int> cands = {0};  // 0: the plain pass
  for (int c = 1; c <= 16; c *= 2)
    if (fits(c)) cands.push_back(c);
  const std::string key = tune_key("lattice_plane_tma", {n1, n2, n_target});
  int nt = 0, st;
  if (in != (const void *)out) {
    auto trial = [&](int v) -> int {
      return v == 0 ? launch_plane<FWD>(in, in_df, out, out_df, outer, n1, n2, n_target, scale, stream)
                    : launch_plane_tma_nt<FWD>(in, in_df, out, out_df, outer, n1, n2, n_target, scale, stream, v);
    };
    st = tune_pick(key, cands, 0, stream, trial, &nt);
  } else {
    st = tune_lookup(key, cands, 0, &nt);  // in place: a trial would transform the data twice
  }
  if (st) return st;
  if (nt == 0) return kNotApplicable;
  return launch_plane_tma_nt<FWD>(in, in_df, out, out_df, outer, n1, n2, n_target, scale, stream, nt);
}

}  // namespace

// Transform over the 3 mesh dims of [n_w, dims..., n_target]; in == out allowed.
__global__ void __launch_bounds__(256) scale_copy_kernel(const double2 *__restrict__ in, double2 *__restrict__ out,
                                                         long n, double s) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = cscale(in[i], s);
}

int launch_lattice_fft(bool forward, long n_w, const int dims[3], long n_target, const double2 *in, double2 *out,
                       cudaStream_t stream) {
  const long nk = (long)dims[0] * dims[1] * dims[2];
  return launch_lattice_fft_scaled(forward, n_w, dims, n_target, in, out, forward ? 1.0 / (double)nk : 1.0, stream);
}

// The lattice transform with an explicit overall factor (the adjoints use the
// unscaled forward and the 1/N_k-scaled backward transforms).
int launch_lattice_fft_scaled(bool forward, long n_w, const int dims[3], long n_target, const double2 *in,
                              double2 *out, double scale_last, cudaStream_t stream) {
  return launch_lattice_fft_fmt(forward, n_w, dims, n_target, in, false, out, false, scale_last, stream);
}

// The general form: input and output each stored as complex128 or (with
// double-float arithmetic) as double-float pairs; the passes in between hand
// each other double-float pairs whenever the arithmetic is double-float.
bool compact_r_to_q_applies(const int dims[3], long n_target) {
  return dims[0] > 1 && dims[1] > 1 && dims[2] > 1 && plane_targets(dims[1], dims[2], n_target) > 0;
}

int launch_lattice_fft_fmt(bool forward, long n_w, const int dims[3], long n_target, const void *in, bool in_df,
                           void *out, bool out_df, double scale_last, cudaStream_t stream, const unsigned *gmax,
                           bool fill_partners, long partner_c, const CompactChi *cc) {
  const bool mid_df = arith_mode() != kArithFP64;
  // with gmax: the n_w = 2 nw - 1 bosonic rows of a real bubble; the first nw - 1
  // (negative frequencies) are left out of the passes, and the last pass stores
  // them from their partners, row j of the others giving row 2 (nw - 1) - j
  const long n_skip = (gmax && n_w >= 3 && (n_w & 1)) ? (n_w - 1) / 2 : 0;
  if (n_skip > 0) {
    fill_partners = true;
    partner_c = 2 * n_skip;
  } else {
    gmax = nullptr;  // partner stores as the caller asks, unconditionally
  }
  int nontriv[3], nn = 0;
  for (int ax = 0; ax < 3; ++ax)
    if (dims[ax] > 1) nontriv[nn++] = ax;
  // the compact canonical orbital columns (CompactChi): the plane pass in place
  // on them, the axis pass from them to every column of `out`
  // (the chain: the rows of both signs with the words, compact rows w = 0 .. nw - 1;
  // a frequency block: its rows w = w0 .. with partner stores at partner_c - row)
  CompactPass cplane = kNoCompact, caxis = kNoCompact;
  if (cc && cc->gmax) {
    const bool whole = gmax && cc->gmax == gmax && n_skip > 0 && cc->rows == n_skip + 1 && cc->w0 == 0;
    const bool block = !gmax && fill_partners && cc->rows == n_w && cc->w0 >= 0;
    if (!(whole || block) || !cc->buf || !cc->oc || !mid_df || !in_df || in != out ||
        !compact_r_to_q_applies(dims, n_target))
      return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: compact columns do not apply to this transform");
    const OrbCanon &oc = *cc->oc;
    const long row0 = whole ? n_skip : 0, prow0 = whole ? n_skip : partner_c;
    const int *kperm = nullptr;
    if (int st = get_k_pair_order(dims[1], dims[2], &kperm)) return st;
    cplane = CompactPass{cc->gmax, cc->buf, cc->rows * dims[0], oc.nc, oc.nc, (int)n_target, 0, 0, 0,
                         oc.ocan, oc.orev, nullptr};
    caxis = CompactPass{cc->gmax, cc->buf, cc->rows, (long)dims[1] * dims[2] * oc.nc, oc.nc, (int)n_target,
                        row0, prow0, cc->w0, oc.ocan, oc.orev, kperm};
  }
  // the partner stores of the last pass, which transforms axis nontriv[0]
  auto mirror_for = [&](int ax) {
    if (!fill_partners) return kNoRowMirror;
    return RowMirror{gmax, partner_c, ax == 0 ? dims[1] : 1, ax <= 1 ? dims[2] : 1, 1};
  };
  if (nn == 0) {  // a single k point: the transform is the identity (times the factor)
    if (in_df || out_df)
      return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: double-float storage needs a mesh with N_k > 1");
    if (fill_partners) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: partner rows need a mesh with N_k > 1");
    const long n = n_w * n_target;
    const double2 *src = static_cast<const double2 *>(in);
    double2 *dst = static_cast<double2 *>(out);
    if (scale_last == 1.0) {
      if (src != dst) TPRF_CUDA(cudaMemcpyAsync(dst, src, n * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
    } else {
      scale_copy_kernel<<<(unsigned)std::min((n + 255) / 256, (long)num_sms() * 8), 256, 0, stream>>>(src, dst, n,
                                                                                                      scale_last);
      TPRF_KERNEL_LAUNCHED("scale_copy_kernel");
    }
    return TPRF_OK;
  }
  // The two fastest-varying non-trivial axes in one pass where they are powers
  // of two; the remaining axis (if any) in a one-axis pass, which then scales.
  if (nn >= 2) {
    const int A = nontriv[nn - 2], B = nontriv[nn - 1];
    if (plane_targets(dims[A], dims[B], n_target) > 0) {
      long outer = n_w;
      for (int a2 = 0; a2 < A; ++a2) outer *= dims[a2];
      const double scale = (nn == 2) ? scale_last : 1.0;
      const bool plane_out_df = (nn == 3) ? mid_df : out_df;
      const SkipRows pskip{gmax, n_skip * (outer / n_w)};
      const RowMirror pmir = (nn == 2) ? mirror_for(A) : kNoRowMirror;
      int st = kNotApplicable;
      if (n_skip == 0 && !pmir.on)  // the TMA form has no row skip and no partner stores
        st = forward ? launch_plane_tma<true>(in, in_df, out, plane_out_df, outer, dims[A], dims[B], n_target, scale,
                                              stream)
                     : launch_plane_tma<false>(in, in_df, out, plane_out_df, outer, dims[A], dims[B], n_target, scale,
                                               stream);
      if (st == kNotApplicable)
        st = forward ? launch_plane<true>(in, in_df, out, plane_out_df, outer, dims[A], dims[B], n_target, scale,
                                          stream, pskip, pmir, cplane)
                     : launch_plane<false>(in, in_df, out, plane_out_df, outer, dims[A], dims[B], n_target, scale,
                                           stream, pskip, pmir, cplane);
      if (st) return st;
      if (nn == 3) {
        const int ax = nontriv[0];
        long outer0 = n_w, inner0 = n_target;
        for (int a2 = 0; a2 < ax; ++a2) outer0 *= dims[a2];
        for (int a2 = ax + 1; a2 < 3; ++a2) inner0 *= dims[a2];
        const SkipRows askip{gmax, n_skip * (outer0 / n_w) * inner0};
        const RowMirror amir = mirror_for(ax);
        st = forward ? launch_axis<true>(out, mid_df, out, out_df, outer0, dims[ax], inner0, scale_last, stream, askip,
                                         amir, caxis)
                     : launch_axis<false>(out, mid_df, out, out_df, outer0, dims[ax], inner0, scale_last, stream,
                                          askip, amir, caxis);
        if (st) return st;
      }
      return TPRF_OK;
    }
  }
  // fastest-varying mesh dimension first: its pass has the longest contiguous rows;
  // the factor on the last pass (the slowest dimension with n > 1)
  const void *src = in;
  bool src_df = in_df;
  for (int i = nn - 1; i >= 0; --i) {
    const int ax = nontriv[i], n = dims[ax];
    long outer = n_w, inner = n_target;
    for (int a2 = 0; a2 < ax; ++a2) outer *= dims[a2];
    for (int a2 = ax + 1; a2 < 3; ++a2) inner *= dims[a2];
    const bool last_pass = (i == 0);
    const double scale = last_pass ? scale_last : 1.0;
    const bool dst_df = last_pass ? out_df : mid_df;
    const SkipRows askip{gmax, n_skip * (outer / n_w) * inner};
    const RowMirror amir = last_pass ? mirror_for(ax) : kNoRowMirror;
    int st = forward ? launch_axis<true>(src, src_df, out, dst_df, outer, n, inner, scale, stream, askip, amir)
                     : launch_axis<false>(src, src_df, out, dst_df, outer, n, inner, scale, stream, askip, amir);
    if (st) return st;
    src = out;
    src_df = dst_df;
  }
  return TPRF_OK;
}

int encode_tensor_map_f64(CUtensorMap *map, const void *base, int rank, const uint64_t *dims,
                          const uint64_t *strides_bytes, const uint32_t *box) {
  static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
  });
  if (!encode) return set_error(TPRF_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  if (rank < 1 || rank > 5 || (reinterpret_cast<uintptr_t>(base) & 15) || (box[0] * 8u) % 16u)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "tensor map: bad rank, base alignment or inner box");
  cuuint64_t gd[5], gs[4];
  cuuint32_t bx[5], es[5];
  for (int i = 0; i < rank; ++i) {
    if (box[i] < 1 || box[i] > 256 || dims[i] < 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "tensor map: box");
    gd[i] = dims[i];
    bx[i] = box[i];
    es[i] = 1;
  }
  for (int i = 0; i + 1 < rank; ++i) {
    if (strides_bytes[i] % 16) return set_error(TPRF_ERR_INVALID_ARGUMENT, "tensor map: stride not a multiple of 16");
    gs[i] = strides_bytes[i];
  }
  const CUresult r = encode(map, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, (cuuint32_t)rank, const_cast<void *>(base), gd, gs,
                            bx, es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return set_error(TPRF_ERR_CUDA, "cuTensorMapEncodeTiled failed: " + std::to_string((int)r));
  return TPRF_OK;
}

}  // namespace tprf

static int check_lattice_args(long n_w, const int dims[3], long n_target, const void *in, const void *out) {
  using namespace tprf;
  if (!dims || !in || !out || n_w < 1 || n_target < 1)
    return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: bad shape or null pointer");
  for (int a = 0; a < 3; ++a)
    if (dims[a] < 1) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: mesh dims must be >= 1");
  return TPRF_OK;
}

extern "C" int tprf_fourier_wk_to_wr(long n_w, const int dims[3], long n_target, const double *g_wk, double *g_wr,
                                     void *stream) {
  int st = check_lattice_args(n_w, dims, n_target, g_wk, g_wr);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  st = tprf::launch_lattice_fft(true, n_w, dims, n_target, reinterpret_cast<const double2 *>(g_wk),
                                reinterpret_cast<double2 *>(g_wr), s);
  if (st) return st;
  TPRF_LAUNCH_CHECK("fourier_wk_to_wr");
  return TPRF_OK;
}

extern "C" int tprf_fourier_wr_to_wk(long n_w, const int dims[3], long n_target, const double *g_wr, double *g_wk,
                                     void *stream) {
  int st = check_lattice_args(n_w, dims, n_target, g_wr, g_wk);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  st = tprf::launch_lattice_fft(false, n_w, dims, n_target, reinterpret_cast<const double2 *>(g_wr),
                                reinterpret_cast<double2 *>(g_wk), s);
  if (st) return st;
  TPRF_LAUNCH_CHECK("fourier_wr_to_wk");
  return TPRF_OK;
}

// ---------------------------------------------------------------------------
// Allocation-free variant of the lattice FFT.
//
// The entry points above keep their FFT tables (twiddles and digit-reversal
// orders, one set per mesh length) in device memory that the library obtains
// with cudaMalloc the first time a length is seen. Some callers cannot let a
// library allocate device memory: codes that hand the whole GPU memory to
// their own pool allocator at start-up and forbid any other device
// allocation, or hosts that run under a fixed, pre-reserved device-memory
// budget. tprf_fourier_lattice_noalloc serves them: its tables live in the
// file-scope array below, which is part of the loaded library image, so no
// call allocates or frees device memory.
//
// Rules of use:
//  * kNoAllocScratchBytes bounds the tables: each distinct mesh length n
//    takes 36 n bytes (plus 256-byte alignment); a transform needing more is
//    refused with TPRF_ERR_INVALID_ARGUMENT before any work is queued.
//  * One CTA transforms whole columns of one mesh axis in shared memory: a
//    mesh length above 12 799 points (6 399 when it has a prime factor above 8)
//    is refused with TPRF_ERR_UNSUPPORTED_SIZE, also before any work.
//  * Every GPU that loads the library holds the array until the process exits.
//  * Every call looks up the array's device address (cudaGetSymbolAddress,
//    which allocates nothing) on the current device, so a device reset cannot
//    leave a stale address behind; the first call on a device may load the
//    library's device code there, so make it before any stream capture.
//  * Every call rebuilds the tables it needs at the start of the array, in
//    stream order before its transform, so nothing from an earlier call is
//    read. Calls that overlap on the GPU (different streams at the same time)
//    share the array and race: serialise them.

namespace tprf {
namespace {

constexpr size_t kNoAllocScratchBytes = 1u << 20;
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// The device address of g_noalloc_scratch on the current device. In host code
// the array's name is only a host-side stand-in; kernels get this address.
int noalloc_scratch_address(unsigned char **out) {
  void *ptr = nullptr;
  cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
  if (e != cudaSuccess) return cuda_status(e, "cudaGetSymbolAddress(g_noalloc_scratch)");
  *out = static_cast<unsigned char *>(ptr);
  return TPRF_OK;
}

// Radix plan of length n (same factor order as the cached plans: 8s, one 4,
// one 2, 3s, 5s, 7s, then larger primes).
bool noalloc_factor(int n, FftDesc *d) {
  int m = n, s = 0;
  while (m % 8 == 0 && s < kMaxStages) { d->radix[s++] = 8; m /= 8; }
  if (m % 4 == 0 && s < kMaxStages) { d->radix[s++] = 4; m /= 4; }
  if (m % 2 == 0 && s < kMaxStages) { d->radix[s++] = 2; m /= 2; }
  for (int r : {3, 5, 7})
    while (m % r == 0 && s < kMaxStages) { d->radix[s++] = r; m /= r; }
  for (int r = 11; (long)r * r <= m && s < kMaxStages; r += 2)
    while (m % r == 0 && s < kMaxStages) { d->radix[s++] = r; m /= r; }
  if (m > 1 && s < kMaxStages) { d->radix[s++] = m; m = 1; }
  d->nst = s;
  d->n = n;
  d->has_generic = 0;
  for (int i = 0; i < s; ++i)
    if (d->radix[i] > 8) d->has_generic = 1;
  return m == 1;
}

size_t noalloc_table_bytes(int n) {
  const size_t b = (size_t)n * (sizeof(double2) + sizeof(float4) + sizeof(int));
  return (b + 255) & ~size_t(255);
}

// Builds the tables of one length in place: twiddles exp(-2 pi i t / n) in FP64
// and as double-float pairs, and the digit-reversal positions.
__global__ void noalloc_tables_kernel(FftDesc d, double2 *tw, float4 *twf, int *rev) {
  const int n = d.n;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    double s, c;
    sincospi(-2.0 * (double)t / (double)n, &s, &c);
    tw[t] = make_double2(c, s);
    const dfl cr = split_double(c), ci = split_double(s);
    twf[t] = make_float4(cr.hi, cr.lo, ci.hi, ci.lo);
    long q = t, prod = 1, sig = 0;
    for (int k = 0; k < d.nst; ++k) {
      const int R = d.radix[k];
      const long dg = q % R;
      q /= R;
      prod *= R;
      sig += dg * (n / prod);
    }
    rev[sig] = t;
  }
}

template <bool FWD, class E>
int noalloc_axis(const double2 *in, double2 *out, long outer, long inner, const FftDesc &d, double scale,
                 cudaStream_t stream) {
  const int n = d.n;
  const int bufs = d.has_generic ? 2 : 1;
  const size_t budget = (size_t)std::min(max_smem_optin(), 200 * 1024);
  int ncol = 64;
  while (ncol > 1 && (size_t)bufs * n * ncol * sizeof(E) + ncol * sizeof(long) > budget) ncol /= 2;
  const long ncols_total = outer * inner;
  while (ncol > 8 && ncol / 2 >= ncols_total) ncol /= 2;
  const size_t smem = (size_t)bufs * n * ncol * sizeof(E) + ncol * sizeof(long);
  int lg = 0;
  while ((1 << lg) < ncol) ++lg;
  const long blocks = (ncols_total + ncol - 1) / ncol;
  auto kern = lattice_axis_kernel<FWD, E, false, false>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  kern<<<(unsigned)blocks, 256, smem, stream>>>(in, out, ncols_total, inner, ncol, lg, d, scale, SkipRows{nullptr, 0},
                                                kNoRowMirror, kNoCompact);
  TPRF_KERNEL_LAUNCHED("lattice_axis_kernel (no-alloc)");
  return TPRF_OK;
}

}  // namespace
}  // namespace tprf

extern "C" int tprf_fourier_lattice_noalloc(int forward, long n_w, const int dims[3], long n_target, const double *in,
                                            double *out, void *stream) {
  using namespace tprf;
  int st = check_lattice_args(n_w, dims, n_target, in, out);
  if (st) return st;
  // tables needed: one set per distinct mesh length > 1, laid out from the start of the array
  int lens[3], nl = 0;
  size_t need = 0;
  for (int ax = 0; ax < 3; ++ax) {
    const int n = dims[ax];
    bool seen = false;
    for (int i = 0; i < nl; ++i) seen |= (lens[i] == n);
    if (n > 1 && !seen) {
      lens[nl++] = n;
      need += noalloc_table_bytes(n);
    }
  }
  if (need > kNoAllocScratchBytes)
    return set_error(TPRF_ERR_INVALID_ARGUMENT,
                     "fourier_lattice_noalloc: FFT tables need " + std::to_string(need) +
                         " bytes, more than the static scratch of " + std::to_string(kNoAllocScratchBytes) +
                         " bytes (36 bytes per point of each distinct mesh length)");
  FftDesc desc[3];
  for (int i = 0; i < nl; ++i)
    if (!noalloc_factor(lens[i], &desc[i]))
      return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "fourier_lattice_noalloc: too many FFT factors");
  for (int i = 0; i < nl; ++i) {
    const size_t bufs = desc[i].has_generic ? 2 : 1;
    if (bufs * (size_t)lens[i] * sizeof(double2) + sizeof(long) > (size_t)std::min(max_smem_optin(), 200 * 1024))
      return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "fourier_lattice_noalloc: mesh dimension too long for one CTA");
  }
  unsigned char *scratch = nullptr;
  st = noalloc_scratch_address(&scratch);
  if (st) return st;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  size_t off = 0;
  for (int i = 0; i < nl; ++i) {
    const int n = lens[i];
    double2 *tw = reinterpret_cast<double2 *>(scratch + off);
    float4 *twf = reinterpret_cast<float4 *>(tw + n);
    int *rev = reinterpret_cast<int *>(twf + n);
    desc[i].tw = tw;
    desc[i].twf = twf;
    desc[i].rev = rev;
    noalloc_tables_kernel<<<(n + 255) / 256, 256, 0, s>>>(desc[i], tw, twf, rev);
    TPRF_KERNEL_LAUNCHED("noalloc_tables_kernel");
    off += noalloc_table_bytes(n);
  }
  const long nk = (long)dims[0] * dims[1] * dims[2];
  const double2 *src = reinterpret_cast<const double2 *>(in);
  double2 *dst = reinterpret_cast<double2 *>(out);
  if (nl == 0) {
    if (src != dst) TPRF_CUDA(cudaMemcpyAsync(dst, src, n_w * n_target * sizeof(double2), cudaMemcpyDeviceToDevice, s));
    return TPRF_OK;
  }
  int first_nontrivial = 0;
  while (dims[first_nontrivial] <= 1) ++first_nontrivial;
  const bool fp64 = arith_mode() == kArithFP64;
  for (int ax = 2; ax >= 0; --ax) {
    const int n = dims[ax];
    if (n <= 1) continue;
    const FftDesc *d = nullptr;
    for (int i = 0; i < nl; ++i)
      if (lens[i] == n) d = &desc[i];
    long outer = n_w, inner = n_target;
    for (int a2 = 0; a2 < ax; ++a2) outer *= dims[a2];
    for (int a2 = ax + 1; a2 < 3; ++a2) inner *= dims[a2];
    const double scale = (forward && ax == first_nontrivial) ? 1.0 / (double)nk : 1.0;
    if (forward)
      st = fp64 ? noalloc_axis<true, double2>(src, dst, outer, inner, *d, scale, s)
                : noalloc_axis<true, cdf>(src, dst, outer, inner, *d, scale, s);
    else
      st = fp64 ? noalloc_axis<false, double2>(src, dst, outer, inner, *d, scale, s)
                : noalloc_axis<false, cdf>(src, dst, outer, inner, *d, scale, s);
    if (st) return st;
    src = dst;
  }
  return TPRF_OK;
}
