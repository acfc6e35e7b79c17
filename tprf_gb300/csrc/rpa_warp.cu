// Kernel (d) for larger vertices (nb >= 4, N = nb^2 >= 16): one warp per
// (w, q) point, the matrix size a runtime value.
//
// Same mathematics as rpa.cu (c++/triqs_tprf/lattice/rpa.cpp:29-64): with the
// particle-hole grouping rows (a, b), columns (d, c), chi = (I - chi0 U)^-1 chi0.
//
// Design: the warp keeps the augmented matrix M = [A | B] (N x 2N, row major,
// A = I - chi0 U, B = chi0) of its point in shared memory. Lanes own columns
// of M, so every row access of the warp touches consecutive 16-byte elements
// (the layout notes at row_ld and group_stride say where conflicts remain).
// Elimination with partial pivoting (pivot search by warp
// shuffles, physical row swaps in A and B) turns A into U and B into L^-1 P B;
// back substitution then runs per B column with no cross-lane dependency. The
// loops are not unrolled over N: one instantiation per element type serves
// every nb, and the code stays small. Double-float by default, with the FP64
// re-solve of points whose conditioning estimate exceeds the double-float
// limit (the estimate of rpa.cu).
#include <algorithm>
#include <climits>
#include <vector>

#include "rpa_common.cuh"

namespace tprf {
namespace {

// the grouped column index of the memory offset m = c' * nb + d inside a row
__device__ __forceinline__ int col_of_offset(int m, int nb) { return (m % nb) * nb + m / nb; }
// grouped column index j -> memory offset of that column inside a row
__device__ __forceinline__ int offset_of_col(int j, int nb) { return (j % nb) * nb + j / nb; }

// U grouped and compacted by columns in shared memory: rows and values, the
// values as the kernel's element type (double-float pairs in the double-float
// kernels, converted once per CTA, so that no solve converts them); an FP64
// solve inside a double-float kernel (the re-solve) reads U itself.
struct SparseU {
  const void *val;     // [nnz] E
  const int *row;
  const int *cs;       // [N + 1] column starts
  const double2 *Ug;   // U in memory order
  bool df;             // val holds double-float pairs
};
template <class E> __device__ __forceinline__ E u_el(const SparseU &u, int t, int c, int N, int nb);
template <>
__device__ __forceinline__ double2 u_el<double2>(const SparseU &u, int t, int c, int N, int nb) {
  return u.df ? u.Ug[u.row[t] * N + offset_of_col(c, nb)] : static_cast<const double2 *>(u.val)[t];
}
template <> __device__ __forceinline__ cdf u_el<cdf>(const SparseU &u, int t, int, int, int) {
  return static_cast<const cdf *>(u.val)[t];
}

// Shared memory of a CTA's compacted U: [N^2] values, [N^2] rows, [N + 1] column starts
__host__ __device__ constexpr size_t sparse_u_bytes(int N) {
  return ((size_t)N * N * (sizeof(double2) + sizeof(int)) + (N + 1) * sizeof(int) + 15) & ~(size_t)15;
}

// Shared-memory layout of a group's augmented matrix [A | B] (N x 2N, 16-byte
// elements; a quarter-warp's 16-byte accesses hit 8 distinct bank quads when
// their element indices differ modulo 8):
//  - rows are row_ld(N) = 2N elements apart. The column accesses (pivot
//    search, scaling of the pivot column, transposed reads) then pair rows i
//    and i + 4 on one quad. An odd stride (2N + 1) removes those conflicts
//    (8.4 % of the shared wavefronts left instead of 15.9 % at nb = 3) but
//    ran 4 % slower on the 32^3 cubic workload with 9 lanes (34.0 against
//    32.6 ms), so the even stride stays;
//  - group_stride(N, G) elements separate the matrices of two groups: N row_ld,
//    padded when a quarter-warp spans two groups (G not a multiple of 8) so that
//    group g starts g * G elements after group 0 modulo 8, and the row
//    accesses of three 9-lane groups cover consecutive quads as one 27-lane
//    group would.
__host__ __device__ constexpr int row_ld(int N) { return 2 * N; }
__host__ __device__ constexpr int group_stride(int N, int G) {
  return (G % 8 == 0) ? N * row_ld(N) : N * row_ld(N) + (((G - N * row_ld(N)) % 8) + 8) % 8;
}

// Pivot magnitudes: float for double-float elements (from the high words; an
// underflow to zero reads as a zero pivot and sends the point to the FP64
// re-solve), double for FP64 elements.
template <class E> struct Mag {
  using type = double;
  static constexpr double big = 1e300;
};
template <> struct Mag<cdf> {
  using type = float;
  static constexpr float big = 3.0e38f;
};
__device__ __forceinline__ double mag2(double2 z) { return cabs2(z); }
__device__ __forceinline__ float mag2(cdf z) { return __fmaf_rn(z.x.hi, z.x.hi, z.y.hi * z.y.hi); }

// Reductions inside a group of G lanes (gmask): xor shuffles when G is a
// power of two, else the warp reduce instructions on order-preserving integer
// keys (non-negative floats and doubles order as their bit patterns). The
// argmax keeps the smallest row index among equal magnitudes; a lane without
// candidate rows (best < 0) takes part with magnitude zero and row j.
constexpr bool pow2_lanes(int g) { return (g & (g - 1)) == 0; }

template <int G>
__device__ __forceinline__ float group_max(float v, unsigned gmask) {
  if constexpr (pow2_lanes(G)) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(gmask, v, o));
    return v;
  } else {
    return __uint_as_float(__reduce_max_sync(gmask, __float_as_uint(fmaxf(v, 0.f))));
  }
}

template <int G, class MagT>
__device__ __forceinline__ void group_argmax(MagT &best, int &p, unsigned gmask) {
  if constexpr (pow2_lanes(G)) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) {
      const MagT ob = __shfl_xor_sync(gmask, best, o);
      const int op = __shfl_xor_sync(gmask, p, o);
      if (ob > best || (ob == best && op < p)) {
        best = ob;
        p = op;
      }
    }
  } else if constexpr (sizeof(MagT) == 4) {
    // one reduction: the magnitude's bits above the low six, then 63 - row (N <= 64),
    // so the largest key is the largest magnitude (to 2^-17 relative, which is all
    // the choice of a pivot needs) with the smallest row among equals
    const unsigned key = (best > 0 ? (__float_as_uint(best) & ~63u) : 0u) | (63u - (unsigned)p);
    const unsigned kmax = __reduce_max_sync(gmask, key);
    p = 63 - (int)(kmax & 63u);
    best = __uint_as_float(kmax & ~63u);
  } else {
    const unsigned long long key = best > 0 ? (unsigned long long)__double_as_longlong(best) : 0ull;
    const unsigned hi = (unsigned)(key >> 32), lo = (unsigned)key;
    const unsigned hmax = __reduce_max_sync(gmask, hi);
    const unsigned lmax = __reduce_max_sync(gmask, hi == hmax ? lo : 0u);
    const unsigned long long kmax = ((unsigned long long)hmax << 32) | lmax;
    p = (int)__reduce_min_sync(gmask, key == kmax ? (unsigned)p : 0xffffffffu);
    best = __longlong_as_double((long long)kmax);
  }
}

// Gaussian elimination with partial pivoting on the group's augmented matrix
// M = [A | B] (N x 2N, rows ld elements apart, shared memory), then back
// substitution: on return the right half holds A^-1 B and the left half the LU
// factors.
// Lanes own columns; the pivot search is a shuffle argmax inside the group.
// Returns the smallest squared pivot magnitude; sets `sing` on a zero pivot.
template <class E, int G, int NC = 0>
__device__ __forceinline__ typename Mag<E>::type solve_augmented(E *M, int N_in, int ld, int lane, unsigned gmask,
                                                                 bool &sing) {
  const int N = NC > 0 ? NC : N_in;  // a compile-time size when NC > 0
  const int W = 2 * N;
#define MM(i, c) M[(i) * ld + (c)]
  using MagT = typename Mag<E>::type;
  MagT pmin = Mag<E>::big;
  for (int j = 0; j < N; ++j) {
    // the updates leave unnormalised double-float values: renormalise the pivot
    // column (read by the search, the reciprocal and the multipliers) and,
    // below, the pivot row (read by the update products)
    for (int i = j + lane; i < N; i += G) MM(i, j) = el_norm(MM(i, j));
    int p = j;
    MagT best = -1;
    for (int i = j + lane; i < N; i += G) {
      const MagT v = mag2(MM(i, j));
      if (v > best) {
        best = v;
        p = i;
      }
    }
    group_argmax<G>(best, p, gmask);
    if (best == 0) sing = true;
    pmin = pmin < best ? pmin : best;
    if (p != j) {
      for (int c = lane; c < W; c += G) {
        const E t = MM(j, c);
        MM(j, c) = MM(p, c);
        MM(p, c) = t;
      }
    }
    __syncwarp(gmask);
    const E inv = el_recip(MM(j, j));
    for (int i = j + 1 + lane; i < N; i += G) MM(i, j) = cmul(MM(i, j), inv);
    __syncwarp(gmask);
    for (int c = j + 1 + lane; c < W; c += G) {
      const E piv = el_norm(MM(j, c));
      MM(j, c) = piv;
#pragma unroll 2
      for (int i = j + 1; i < N; ++i) MM(i, c) = el_fms_lazy(MM(i, j), piv, MM(i, c));
    }
    __syncwarp(gmask);
    if (lane == 0) MM(j, j) = inv;
    __syncwarp(gmask);
  }
  // back substitution, one B column per lane (B renormalised as it is read)
  for (int c = N + lane; c < W; c += G) {
    for (int j = N - 1; j >= 0; --j) {
      const E xj = cmul(el_norm(MM(j, c)), MM(j, j));
      MM(j, c) = xj;
#pragma unroll 2
      for (int i = 0; i < j; ++i) MM(i, c) = el_fms_lazy(MM(i, j), xj, MM(i, c));
    }
  }
  __syncwarp(gmask);
#undef MM
  return pmin;
}

// b_ready: the caller has already written B = chi0 (from x) into M, with the
// same lane of the group writing element o as the load loop here would.
template <class E, int G, int NBC = 0>
__device__ typename Mag<E>::type rpa_point_warp(const double2 *__restrict__ x, double2 *__restrict__ y, E *M, int N_in, int nb_in,
                                 const SparseU &u, int lane, unsigned gmask, bool &singular,
                                 double2 *__restrict__ y_conj = nullptr, bool b_ready = false) {
  const int nb = NBC > 0 ? NBC : nb_in;  // a compile-time size when NBC > 0
  const int N = NBC > 0 ? NBC * NBC : N_in;
  const int LD = row_ld(N);
#define MM(i, c) M[(i) * LD + (c)]
  // B = chi0 in the grouped layout (coalesced global reads)
  if (!b_ready)
    for (int o = lane; o < N * N; o += G) MM(o / N, N + col_of_offset(o % N, nb)) = el_from(x[o], (E *)nullptr);
  __syncwarp(gmask);
  // A = I - X U from the non-zeros of U; the size of the terms bounds cancellation
  float amax = 0.f;
  for (int e = lane; e < N * N; e += G) {
    const int r = e / N, c = e % N;
    E s = (r == c) ? el_one((E *)nullptr) : el_zero((E *)nullptr);
    float mag = (r == c) ? 1.f : 0.f;
    for (int t = u.cs[c]; t < u.cs[c + 1]; ++t) {
      const E xv = MM(r, N + u.row[t]);
      const E uv = u_el<E>(u, t, c, N, nb);
      s = el_fms(xv, uv, s);
      mag = fmaf(el_absf(xv), el_absf(uv), mag);
    }
    amax = fmaxf(amax, mag);
    MM(r, c) = s;
  }
  __syncwarp(gmask);
#undef MM
  bool sing = false;
  const auto pmin = solve_augmented<E, G, NBC * NBC>(M, N, LD, lane, gmask, sing);
  singular = sing;
  for (int o = lane; o < N * N; o += G) {
    const double2 v = el_to(M[(o / N) * LD + N + col_of_offset(o % N, nb)]);
    y[o] = v;
    if (y_conj) y_conj[o] = make_double2(v.x, -v.y);  // the solve of the conjugate system, bit for bit
  }
  amax = group_max<G>(amax, gmask);
  __syncwarp(gmask);
  if constexpr (IsDf<E>::value) {
    // in float: the estimate only meets the re-solve limit and the transpose
    // test, and the FP64 pipe stays free of per-point bookkeeping
    return pmin > 0.f ? amax * amax / pmin : INFINITY;
  } else {
    const double am = (double)amax * (double)amax;
    return pmin > 0 ? am / (double)pmin : 1e300;
  }
}


// The FP64 re-solve of a double-float point, out of line: it runs for points
// near an instability only, and inlined its register demand would shape the
// allocation (and the spills) of the double-float solve around it.
template <int G, int NBC>
__device__ __noinline__ void resolve_fp64(const double2 *x, double2 *y, double2 *M, int N, int nb, const SparseU &u,
                                          int lane, unsigned gmask, bool &singular, double2 *y_conj) {
  rpa_point_warp<double2, G, NBC>(x, y, M, N, nb, u, lane, gmask, singular, y_conj);
}

template <class E, int G, int NBC = 0>
__global__ void __launch_bounds__(512) rpa_warp_kernel(long n_points, int nb_in, const double2 *__restrict__ chi0,
                                                       const double2 *__restrict__ U, double2 *__restrict__ chi,
                                                       unsigned *status) {
  const int nb = NBC > 0 ? NBC : nb_in;
  const int N = nb * nb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *s_val = reinterpret_cast<double2 *>(smem_raw);
  int *s_row = reinterpret_cast<int *>(s_val + N * N);
  int *s_cs = s_row + N * N;
  const size_t u_bytes = sparse_u_bytes(N);
  // groups of G lanes, one point per group, 32 / G groups in each warp (the
  // lanes past the last whole group of a warp stay idle)
  constexpr int GPW = 32 / G;
  const int wl = threadIdx.x & 31, gw = wl / G;
  const int grp = (threadIdx.x >> 5) * GPW + gw, lane = wl - gw * G, n_grp = (blockDim.x >> 5) * GPW;
  const bool active = gw < GPW;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (gw * G));
  E *M = reinterpret_cast<E *>(smem_raw + u_bytes) + (size_t)(active ? grp : 0) * group_stride(N, G);
  if (threadIdx.x == 0) {
    int t = 0;
    for (int c = 0; c < N; ++c) {
      s_cs[c] = t;
      for (int m = 0; m < N; ++m) {
        // grouped U[m][c] = U_{m_a m_b, c_d c_c}: memory offset m * N + offset(c)
        const double2 v = U[m * N + (c % nb) * nb + c / nb];
        if (v.x != 0.0 || v.y != 0.0) {
          s_row[t] = m;
          s_val[t] = v;
          ++t;
        }
      }
    }
    s_cs[N] = t;
  }
  __syncthreads();
  if constexpr (IsDf<E>::value) {  // the values in the element type, in place
    for (int t = threadIdx.x; t < s_cs[N]; t += blockDim.x) {
      const double2 v = s_val[t];
      reinterpret_cast<cdf *>(s_val)[t] = to_cdf(v);
    }
    __syncthreads();
  }
  const SparseU u{s_val, s_row, s_cs, U, IsDf<E>::value};
  if (!active) return;
  for (long pt = (long)blockIdx.x * n_grp + grp; pt < n_points; pt += (long)gridDim.x * n_grp) {
    const double2 *x = chi0 + pt * N * N;
    double2 *y = chi + pt * N * N;
    bool singular = false;
    const auto cond2 = rpa_point_warp<E, G, NBC>(x, y, M, N, nb, u, lane, gmask, singular);
    if (IsDf<E>::value && !(cond2 <= (typename Mag<E>::type)kDf64CondLimit2))
      resolve_fp64<G, NBC>(x, y, reinterpret_cast<double2 *>(M), N, nb, u, lane, gmask, singular, nullptr);
    if (singular && lane == 0) atomicOr(status, kDevErrSingular);
  }
}

// Conjugate pairs on a bosonic (w, q) mesh: with U real, chi0(-w, q) =
// conj(chi0(w, -q)) (a real bubble gives this exactly) makes A(-w, q) the
// conjugate of A(w, -q), and the elimination (conjugation only flips signs,
// which every step preserves) gives chi(-w, q) = conj(chi(w, -q)) bit for bit.
//
// Transposition partners: with real hoppings, G(tau, -r) = G(tau, r)^T, so the
// grouped chi0(w, -q) is the transpose of chi0(w, q); with a symmetric grouped
// U (Kanamori vertices are), chi(w, -q) = chi(w, q)^T as well (push-through:
// (I - X^T U)^-1 X^T = [X (I - U X)^-1]^T = [(I - X U)^-1 X]^T). The computed
// chi0 meets the symmetry to rounding only, so the transpose stands in for the
// direct solve of (w, -q) when the asymmetry d = max |chi0(w, -q) -
// chi0(w, q)^T| is small against the solve's conditioning estimate k:
// d k <= kTransposeTol max |chi0(w, q)|; the transposed result then lies within
// that bound of a direct solve. Otherwise (w, -q) is solved on its own. Never in
// the FP64 mode, which solves every point as the plain path.
//
// A group takes a unit (w >= 0, q) and its partners: (-w, -q) (conjugate) and,
// for w > 0, q != -q and a symmetric U, also (w, -q) (transpose) and (-w, q)
// (its conjugate). Units: w = 0 with q <= -q; w > 0 with q <= -q when
// transposes are allowed, else every q.
constexpr float kTransposeTol2 = 1e-24f;  // kTransposeTol = 1e-12, squared

// max(|Re(a - b)|, |Im(a - b)|) and max(|Re a|, |Im a|) as floats
__device__ __forceinline__ float el_max_abs(double2 a) { return (float)fmax(fabs(a.x), fabs(a.y)); }
__device__ __forceinline__ float el_max_abs(cdf a) { return fmaxf(fabsf(a.x.hi), fabsf(a.y.hi)); }

// B = chi0 of the point at x written to the group's matrix M (as rpa_point_warp
// would), and whether the point at xc holds its conjugate bit for bit (with
// U real; only when test)
template <class E, int G>
__device__ __forceinline__ bool load_b_conj(const double2 *__restrict__ x, const double2 *__restrict__ xc, bool test,
                                            bool ureal, E *M, int N, int nb, int lane, unsigned gmask) {
  bool sym = ureal;
  for (int o = lane; o < N * N; o += G) {
    const double2 a = x[o];
    M[(o / N) * row_ld(N) + N + col_of_offset(o % N, nb)] = el_from(a, (E *)nullptr);
    if (test) {
      const double2 b = xc[o];
      sym = sym && __double_as_longlong(a.x) == __double_as_longlong(b.x) &&
            __double_as_longlong(a.y) == __double_as_longlong(-b.y);
    }
  }
  return test && __all_sync(gmask, sym);
}

// One point solve (B already in M when b_ready) writing chi to ys and, when yc
// is given, its conjugate to yc; the FP64 re-solve when the conditioning
// estimate asks for it. Returns the squared estimate (float) and whether the
// solution left in M is the FP64 one.
struct PairSolve {
  float cond2;
  bool in64;
};
template <class E, int G, int NBC>
__device__ __forceinline__ PairSolve solve_pair_point(const double2 *xs, double2 *ys, double2 *yc, bool b_ready, E *M,
                                                      int N, int nb, const SparseU &u, int lane, unsigned gmask,
                                                      unsigned *status) {
  bool singular = false;
  PairSolve r{(float)rpa_point_warp<E, G, NBC>(xs, ys, M, N, nb, u, lane, gmask, singular, yc, b_ready), false};
  if (IsDf<E>::value && !(r.cond2 <= (float)kDf64CondLimit2)) {
    resolve_fp64<G, NBC>(xs, ys, reinterpret_cast<double2 *>(M), N, nb, u, lane, gmask, singular, yc);
    r.in64 = true;
  }
  if (singular && lane == 0) atomicOr(status, kDevErrSingular);
  return r;
}

// 448 threads and two CTAs per SM: a 72-register budget. Measured on the
// 32^3 cubic workload (nb = 3, 9 lanes): 32.6 ms, against 34.7 ms at 80
// registers (384 threads), 36.2 ms at 64 (512 threads, some spills) and
// 42.4 ms unbounded (102 registers, 19 warps per SM).
template <class E, int G, int NBC = 0>
__global__ void __launch_bounds__(448, 2) rpa_pair_kernel(int nw, int d0, int d1, int d2, int nb_in,
                                                       const double2 *__restrict__ chi0, const double2 *__restrict__ U,
                                                       PairOut out, unsigned *status) {
  const int nb = NBC > 0 ? NBC : nb_in;
  const int N = nb * nb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *s_val = reinterpret_cast<double2 *>(smem_raw);
  int *s_row = reinterpret_cast<int *>(s_val + N * N);
  int *s_cs = s_row + N * N;
  __shared__ int s_ureal, s_usym;
  const size_t u_bytes = sparse_u_bytes(N);
  constexpr int GPW = 32 / G;
  const int wl = threadIdx.x & 31, gw = wl / G;
  const int grp = (threadIdx.x >> 5) * GPW + gw, lane = wl - gw * G, n_grp = (blockDim.x >> 5) * GPW;
  const bool active = gw < GPW;
  const unsigned gmask = (G == 32) ? 0xffffffffu : (((1u << G) - 1u) << (gw * G));
  E *M = reinterpret_cast<E *>(smem_raw + u_bytes) + (size_t)(active ? grp : 0) * group_stride(N, G);
  if (threadIdx.x == 0) {
    int t = 0, ureal = 1, usym = 1;
    for (int c = 0; c < N; ++c) {
      s_cs[c] = t;
      for (int m = 0; m < N; ++m) {
        // grouped U[m][c] at memory offset m * N + offset(c); symmetric: U[m][c] == U[c][m]
        const double2 v = U[m * N + offset_of_col(c, nb)], vt = U[c * N + offset_of_col(m, nb)];
        if (v.y != 0.0) ureal = 0;
        if (__double_as_longlong(v.x) != __double_as_longlong(vt.x) ||
            __double_as_longlong(v.y) != __double_as_longlong(vt.y))
          usym = 0;
        if (v.x != 0.0 || v.y != 0.0) {
          s_row[t] = m;
          s_val[t] = v;
          ++t;
        }
      }
    }
    s_cs[N] = t;
    s_ureal = ureal;
    s_usym = usym;
  }
  __syncthreads();
  if constexpr (IsDf<E>::value) {  // the values in the element type, in place
    for (int t = threadIdx.x; t < s_cs[N]; t += blockDim.x) {
      const double2 v = s_val[t];
      reinterpret_cast<cdf *>(s_val)[t] = to_cdf(v);
    }
    __syncthreads();
  }
  const SparseU u{s_val, s_row, s_cs, U, IsDf<E>::value};
  const bool ureal = s_ureal != 0;
  const bool tpairs = s_usym != 0 && IsDf<E>::value;  // transposition partners (never in the FP64 mode)
  if (!active) return;
  // fewer than 2^31 units per launch (launch_pair_as splits larger frequency
  // ranges): 32-bit index arithmetic, no 64-bit division
  const unsigned nk = (unsigned)d0 * d1 * d2, d12 = (unsigned)d1 * d2, units = (unsigned)(out.mh1 - out.mh0) * nk;
  for (unsigned un = blockIdx.x * n_grp + grp; un < units; un += gridDim.x * n_grp) {
    const unsigned fm = un / nk, qu = un - fm * nk;
    const int mh = out.mh0 + (int)fm;
    const long q = qu;
    const unsigned q0 = qu / d12, r12 = qu - q0 * d12, q1 = r12 / d2, q2 = r12 - q1 * d2;
    const long mq = ((long)((d0 - q0) % d0) * d1 + (d1 - q1) % d1) * d2 + (d2 - q2) % d2;
    if (q > mq && (mh == 0 || tpairs)) continue;  // a partner's unit holds this point
    // the unit's points: 0 = (w, q), 1 = (-w, -q) its conjugate, and for a
    // transposition unit 2 = (w, -q), 3 = (-w, q) its conjugate; each point's
    // chi0 is read once
    const long p0 = (long)(nw - 1 + mh) * nk + q, p1 = (long)(nw - 1 - mh) * nk + mq;
    const bool quad = tpairs && mh > 0 && q < mq;
    double2 *const row_pos = out.pos + (long)(mh - out.mh0) * out.row;
    double2 *const row_neg = mh == 0 ? row_pos : out.neg + (long)(mh - out.mh0) * out.neg_step;
    const bool done1 = p1 == p0;
    // point 0 into B (with the conjugate test against point 1)
    const bool sym = load_b_conj<E, G>(chi0 + p0 * N * N, chi0 + p1 * N * N, !done1, ureal, M, N, nb, lane, gmask);
    __syncwarp(gmask);
    // a quad: point 2 against the transpose of point 0's B (in the element type;
    // bit-equal inputs give bit-equal elements), and the conjugate test of point 3
    float dmax = 0.f, amax = 0.f;
    bool sym3 = false;
    if (quad) {
      const double2 *x0 = chi0 + p0 * N * N;
      const double2 *x2 = chi0 + ((long)(nw - 1 + mh) * nk + mq) * N * N;
      const double2 *x3 = chi0 + ((long)(nw - 1 - mh) * nk + q) * N * N;
      bool s3 = ureal;
      // the largest |chi0(w, -q) - chi0(w, q)^T| in FP64, kept as the bits of a
      // non-negative double (which order as integers; a NaN difference sorts above
      // every number and refuses the transpose)
      unsigned long long dbits = 0ull;
      for (int o = lane; o < N * N; o += G) {
        const int i = o / N, j = col_of_offset(o % N, nb);
        const double2 b = x2[o], c = x3[o];
        s3 = s3 && __double_as_longlong(b.x) == __double_as_longlong(c.x) &&
             __double_as_longlong(b.y) == __double_as_longlong(-c.y);
        const double2 a0 = x0[j * N + offset_of_col(i, nb)];  // chi0(w, q)[j][i], as loaded into B
        const unsigned long long dx = (unsigned long long)__double_as_longlong(__dsub_rn(b.x, a0.x)) & ~(1ull << 63);
        const unsigned long long dy = (unsigned long long)__double_as_longlong(__dsub_rn(b.y, a0.y)) & ~(1ull << 63);
        dbits = dbits > dx ? dbits : dx;
        dbits = dbits > dy ? dbits : dy;
        amax = fmaxf(amax, el_max_abs(M[j * row_ld(N) + N + i]));
      }
      sym3 = __all_sync(gmask, s3);
      const double dm = __longlong_as_double((long long)dbits);
      dmax = dm != dm ? INFINITY : __double2float_ru(dm);  // rounded up: the test stays conservative
      dmax = group_max<G>(dmax, gmask);
      amax = group_max<G>(amax, gmask);
    }
    const PairSolve s0 = solve_pair_point<E, G, NBC>(chi0 + p0 * N * N, row_pos + q * N * N,
                                                     sym ? row_neg + mq * N * N : nullptr, true, M, N, nb, u, lane,
                                                     gmask, status);
    // chi(w, -q) = chi(w, q)^T when chi0(w, -q) is chi0(w, q)^T to within the
    // solve's conditioning (the transposed solution is read from M); in float
    // (a threshold test: underflow of amax^2 only refuses the transpose)
    const bool take_t =
        quad && s0.cond2 < INFINITY && dmax * dmax * s0.cond2 <= kTransposeTol2 * amax * amax;
    if (take_t) {
      const bool in64 = s0.in64;  // the solution left in M is the FP64 one
      double2 *y2 = row_pos + mq * N * N, *y3 = row_neg + q * N * N;
      for (int o = lane; o < N * N; o += G) {
        const int i = o / N, j = col_of_offset(o % N, nb);
        const int at = j * row_ld(N) + N + i;
        const double2 v = in64 ? reinterpret_cast<const double2 *>(M)[at] : el_to(M[at]);
        y2[o] = v;
        if (sym3) y3[o] = make_double2(v.x, -v.y);
      }
      __syncwarp(gmask);
    }
    if (!sym && !done1)
      solve_pair_point<E, G, NBC>(chi0 + p1 * N * N, row_neg + mq * N * N, nullptr, false, M, N, nb, u, lane, gmask,
                                  status);
    if (quad && !(take_t && sym3)) {
      // point 3 on its own (transpose taken, no conjugate), or points 2 and 3
      const long p2 = (long)(nw - 1 + mh) * nk + mq, p3 = (long)(nw - 1 - mh) * nk + q;
      bool sym2 = false;
      if (!take_t) {
        sym2 = load_b_conj<E, G>(chi0 + p2 * N * N, chi0 + p3 * N * N, true, ureal, M, N, nb, lane, gmask);
        __syncwarp(gmask);
        solve_pair_point<E, G, NBC>(chi0 + p2 * N * N, row_pos + mq * N * N, sym2 ? row_neg + q * N * N : nullptr,
                                    true, M, N, nb, u, lane, gmask, status);
      }
      if (!sym2)
        solve_pair_point<E, G, NBC>(chi0 + p3 * N * N, row_neg + q * N * N, nullptr, false, M, N, nb, u, lane, gmask,
                                    status);
    }
  }
}

template <class E, int G, int NBC = 0>
int launch_as(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
              unsigned *status) {
  const int N = nb * nb;
  const size_t u_bytes = sparse_u_bytes(N);
  const size_t per_point = (size_t)group_stride(N, G) * 16;
  const int ppw = 32 / G;  // points per warp
  const size_t limit = (size_t)max_smem_optin();
  if (u_bytes + ppw * per_point > limit) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  TPRF_CUDA(cudaFuncSetAttribute(rpa_warp_kernel<E, G, NBC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
  // the number of warps per CTA that puts the most warps on an SM
  int best_w = 1, best_total = 0;
  for (int w = 1; w <= 16; ++w) {
    const size_t smem = u_bytes + (size_t)w * ppw * per_point;
    if (smem > limit) break;
    int per_sm = 0;
    TPRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rpa_warp_kernel<E, G, NBC>, 32 * w, smem));
    if (per_sm * w >= best_total) {
      best_total = per_sm * w;
      best_w = w;
    }
  }
  if (best_total == 0) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  const size_t smem = u_bytes + (size_t)best_w * ppw * per_point;
  const long per_block = (long)best_w * ppw;
  long blocks = (n_points + per_block - 1) / per_block;
  blocks = std::max(1L, std::min(blocks, (long)num_sms() * (best_total / best_w) * 8));
  rpa_warp_kernel<E, G, NBC><<<(unsigned)blocks, 32 * best_w, smem, stream>>>(n_points, nb, chi0, U, chi, status);
  TPRF_KERNEL_LAUNCHED("rpa_warp_kernel");
  return TPRF_OK;
}

// Sizes compiled in full: nb = 3 (9 x 9) and nb = 5 (25 x 25); other vertex
// sizes run the runtime-sized form of the same kernel.
template <int G>
int launch_g(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
             unsigned *status) {
  const bool fp64 = arith_mode() == kArithFP64;
  if (nb == 3)
    return fp64 ? launch_as<double2, G, 3>(n_points, nb, chi0, U, chi, stream, status)
                : launch_as<cdf, G, 3>(n_points, nb, chi0, U, chi, stream, status);
  if (nb == 5 && G >= 16)
    return fp64 ? launch_as<double2, G, 5>(n_points, nb, chi0, U, chi, stream, status)
                : launch_as<cdf, G, 5>(n_points, nb, chi0, U, chi, stream, status);
  return fp64 ? launch_as<double2, G>(n_points, nb, chi0, U, chi, stream, status)
              : launch_as<cdf, G>(n_points, nb, chi0, U, chi, stream, status);
}

// ---- screened interaction W ---------------------------------------------------------
// dynamical_screened_interaction.cpp, per (w, k) point, on PH-grouped matrices
// (rows (a,b), columns (d,c)) with S the pair swap (e,f) <-> (f,e):
//   static V(k) (:85-124): D(a,b,c,d) = delta_ad delta_bc - sum_ef PI(a,b,e,f) V(e,f,c,d)
//     is D = I - PI S V, and W(a,b,c,d) = sum_ef V(a,b,e,f) D^-1(e,f,c,d) is W = V S D^-1;
//   dynamic V(w, k) (:30-80): W = V (I - PI V)^-1, the same with S = I.
// W D = V S, so the group solves D^T W^T = S V^T: [D^T | S V^T] in shared memory,
// FP64, then stores W transposed back. One warp per point.
__device__ __forceinline__ int pair_swap(int m, int nb) { return (m % nb) * nb + m / nb; }

__global__ void __launch_bounds__(256) screened_w_kernel(long n_points, long nk, int nb, int swap, int v_per_point,
                                                         const double2 *__restrict__ PI,
                                                         const double2 *__restrict__ V, double2 *__restrict__ Wout,
                                                         unsigned *status) {
  const int N = nb * nb;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, n_warps = blockDim.x >> 5;
  double2 *M = reinterpret_cast<double2 *>(smem_raw) + (size_t)warp * 4 * N * N;
  double2 *P = M + 2 * N * N, *Vg = P + N * N;  // PI and V in the grouped layout
  for (long pt = (long)blockIdx.x * n_warps + warp; pt < n_points; pt += (long)gridDim.x * n_warps) {
    const double2 *pi = PI + pt * N * N;
    const double2 *v = V + (v_per_point ? pt : pt % nk) * N * N;
    for (int o = lane; o < N * N; o += 32) {
      const int r = o / N, gc = col_of_offset(o % N, nb);
      P[r * N + gc] = pi[o];
      Vg[r * N + gc] = v[o];
    }
    __syncwarp();
    for (int e = lane; e < N * N; e += 32) {
      const int i = e / N, j = e % N;
      double2 s = make_double2(i == j ? 1.0 : 0.0, 0.0);
      for (int m = 0; m < N; ++m) s = cfms(P[j * N + (swap ? pair_swap(m, nb) : m)], Vg[m * N + i], s);
      M[i * 2 * N + j] = s;                                                // D^T[i][j]
      M[i * 2 * N + N + j] = Vg[j * N + (swap ? pair_swap(i, nb) : i)];  // (S V^T)[i][j]
    }
    __syncwarp();
    bool sing = false;
    solve_augmented<double2, 32>(M, N, 2 * N, lane, 0xffffffffu, sing);
    if (sing && lane == 0) atomicOr(status, kDevErrSingular);
    double2 *w = Wout + pt * N * N;
    for (int o = lane; o < N * N; o += 32) {
      const int r = o / N, gc = col_of_offset(o % N, nb);
      w[o] = M[gc * 2 * N + N + r];  // W[r][gc] = (W^T)[gc][r]
    }
    __syncwarp();
  }
}

// ---- adjoint -------------------------------------------------------------------
// With A = I - X0 U (grouped) and X = A^-1 X0: d X = A^-1 dX0 (I + U X) + X dU X.
// For a real loss with conjugate-Wirtinger gradient Y = dL/dX:
//   X0_grad = Z B^H with A^H Z = Y and B = I + U X,
//   U_grad  = sum over points of X^H Y X^H.
// One warp per point in FP64. Per warp, shared memory holds [A^H | Y] (N x 2N,
// eliminated in place into [U | Z]), X, a copy of Y and the warp's U_grad
// accumulator (each lane owns its entries, so no atomics inside the warp); the
// CTA adds its warps' accumulators into U_grad with one atomic per entry.
__device__ __forceinline__ int grouped_offset(int c, int nb) { return (c % nb) * nb + c / nb; }

__global__ void __launch_bounds__(512) rpa_adjoint_warp_kernel(long n_points, int nb, const double2 *__restrict__ chi0,
                                                               const double2 *__restrict__ U,
                                                               const double2 *__restrict__ chi,
                                                               const double2 *__restrict__ chig,
                                                               double2 *__restrict__ chi0g, double2 *Ug,
                                                               unsigned *status) {
  const int N = nb * nb, W = 2 * N;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  double2 *s_val = reinterpret_cast<double2 *>(smem_raw);
  int *s_row = reinterpret_cast<int *>(s_val + N * N);
  int *s_col = s_row + N * N;
  int *s_cs = s_col + N * N;
  const size_t u_bytes =
      ((size_t)N * N * (sizeof(double2) + 2 * sizeof(int)) + (N + 1) * sizeof(int) + 15) & ~(size_t)15;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, n_warps = blockDim.x >> 5;
  double2 *M = reinterpret_cast<double2 *>(smem_raw + u_bytes) + (size_t)warp * 5 * N * N;
  double2 *Xs = M + 2 * N * N, *Yc = Xs + N * N, *Acc = Yc + N * N;
  if (threadIdx.x == 0) {
    int t = 0;
    for (int c = 0; c < N; ++c) {
      s_cs[c] = t;
      for (int m = 0; m < N; ++m) {
        const double2 v = U[m * N + grouped_offset(c, nb)];
        if (v.x != 0.0 || v.y != 0.0) {
          s_row[t] = m;
          s_col[t] = c;
          s_val[t] = v;
          ++t;
        }
      }
    }
    s_cs[N] = t;
  }
  for (int e = lane; e < N * N; e += 32) Acc[e] = make_double2(0.0, 0.0);
  __syncthreads();
  const int nnz = s_cs[N];
#define MM(i, c) M[(i) * W + (c)]
  for (long pt = (long)blockIdx.x * n_warps + warp; pt < n_points; pt += (long)gridDim.x * n_warps) {
    const long o = pt * N * N;
    for (int e = lane; e < N * N; e += 32) {
      const int r = e / N, c = col_of_offset(e % N, nb);
      Xs[r * N + c] = chi[o + e];
      const double2 y = chig[o + e];
      Yc[r * N + c] = y;
      MM(r, N + c) = y;
    }
    // A^H[i][j] = delta_ij - sum_m conj(U[m][i]) conj(X0[j][m]), U's column i
    for (int e = lane; e < N * N; e += 32) {
      const int i = e / N, j = e % N;
      double2 s = make_double2(i == j ? 1.0 : 0.0, 0.0);
      for (int t = s_cs[i]; t < s_cs[i + 1]; ++t)
        s = cfms(cconj(s_val[t]), cconj(chi0[o + j * N + grouped_offset(s_row[t], nb)]), s);
      MM(i, j) = s;
    }
    __syncwarp();
    bool sing = false;
    for (int j = 0; j < N; ++j) {
      int p = j;
      double best = -1.0;
      for (int i = j + lane; i < N; i += 32) {
        const double v = cabs2(MM(i, j));
        if (v > best) {
          best = v;
          p = i;
        }
      }
#pragma unroll
      for (int off = 16; off > 0; off >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, off);
        const int op = __shfl_xor_sync(0xffffffffu, p, off);
        if (ob > best || (ob == best && op < p)) {
          best = ob;
          p = op;
        }
      }
      if (best == 0.0) sing = true;
      if (p != j)
        for (int c = lane; c < W; c += 32) {
          const double2 t = MM(j, c);
          MM(j, c) = MM(p, c);
          MM(p, c) = t;
        }
      __syncwarp();
      const double2 inv = crecip(MM(j, j));
      for (int i = j + 1 + lane; i < N; i += 32) MM(i, j) = cmul(MM(i, j), inv);
      __syncwarp();
      for (int c = j + 1 + lane; c < W; c += 32) {
        const double2 piv = MM(j, c);
        for (int i = j + 1; i < N; ++i) MM(i, c) = cfms(MM(i, j), piv, MM(i, c));
      }
      __syncwarp();
      if (lane == 0) MM(j, j) = inv;
      __syncwarp();
    }
    for (int c = N + lane; c < W; c += 32)
      for (int j = N - 1; j >= 0; --j) {
        const double2 zj = cmul(MM(j, c), MM(j, j));
        MM(j, c) = zj;
        for (int i = 0; i < j; ++i) MM(i, c) = cfms(MM(i, j), zj, MM(i, c));
      }
    __syncwarp();
    if (sing && lane == 0) atomicOr(status, kDevErrSingular);
    // B = I + U X into the left half (lane owns column l)
    for (int l = lane; l < N; l += 32) {
      for (int r = 0; r < N; ++r) MM(r, l) = make_double2(r == l ? 1.0 : 0.0, 0.0);
      for (int t = 0; t < nnz; ++t) MM(s_row[t], l) = cfma(s_val[t], Xs[s_col[t] * N + l], MM(s_row[t], l));
    }
    __syncwarp();
    // X0_grad[i][j] = sum_l Z[i][l] conj(B[j][l])
    for (int e = lane; e < N * N; e += 32) {
      const int i = e / N, j = e % N;
      double2 s = make_double2(0.0, 0.0);
      for (int l = 0; l < N; ++l) s = cfma(MM(i, N + l), cconj(MM(j, l)), s);
      chi0g[o + i * N + grouped_offset(j, nb)] = s;
    }
    __syncwarp();
    // T = Y X^H into the left half, then Acc += X^H T
    for (int e = lane; e < N * N; e += 32) {
      const int l = e / N, j = e % N;
      double2 s = make_double2(0.0, 0.0);
      for (int m = 0; m < N; ++m) s = cfma(Yc[l * N + m], cconj(Xs[j * N + m]), s);
      MM(l, j) = s;
    }
    __syncwarp();
    for (int e = lane; e < N * N; e += 32) {
      const int i = e / N, j = e % N;
      double2 s = Acc[e];
      for (int l = 0; l < N; ++l) s = cfma(cconj(Xs[l * N + i]), MM(l, j), s);
      Acc[e] = s;
    }
    __syncwarp();
  }
#undef MM
  __syncthreads();
  for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
    double2 s = make_double2(0.0, 0.0);
    for (int w = 0; w < n_warps; ++w) {
      const double2 *a = reinterpret_cast<double2 *>(smem_raw + u_bytes) + (size_t)w * 5 * N * N + 4 * N * N;
      s = cadd(s, a[e]);
    }
    // grouped (m, c) -> tensor offset m * N + offset(c)
    const int off = (e / N) * N + grouped_offset(e % N, nb);
    atomicAdd(&reinterpret_cast<double *>(Ug)[2 * off], s.x);
    atomicAdd(&reinterpret_cast<double *>(Ug)[2 * off + 1], s.y);
  }
}

}  // namespace

// lanes per point (measured on GB300 with the compiled sizes: nb = 3 9 lanes,
// 32.6 ms for the 16.7 M points of the 32^3 cubic workload in conjugate and
// transposition partners, against 34.0 ms with 8 and 33.7 ms with 16;
// nb = 5 32 lanes, 248 ms for 2.1 M points, against 376 ms with 16)
int rpa_group_lanes(int nb) { return nb <= 2 ? 8 : nb == 3 ? 9 : 32; }

template <class E, int G, int NBC>
int launch_pair_as(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, PairOut out,
                   cudaStream_t stream, unsigned *status) {
  const int N = nb * nb;
  const size_t u_bytes = sparse_u_bytes(N);
  const size_t per_point = (size_t)group_stride(N, G) * 16;
  const int ppw = 32 / G;
  const size_t limit = (size_t)max_smem_optin() - 64;  // the kernel's static word
  if (u_bytes + ppw * per_point > limit) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  auto kern = rpa_pair_kernel<E, G, NBC>;
  TPRF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
  cudaFuncAttributes fa{};
  TPRF_CUDA(cudaFuncGetAttributes(&fa, kern));
  int best_w = 1, best_total = 0;
  for (int w = 1; w <= std::min(16, fa.maxThreadsPerBlock / 32); ++w) {
    const size_t smem = u_bytes + (size_t)w * ppw * per_point;
    if (smem > limit) break;
    int per_sm = 0;
    TPRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 32 * w, smem));
    if (per_sm * w >= best_total) {
      best_total = per_sm * w;
      best_w = w;
    }
  }
  if (best_total == 0) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: nb too large");
  const size_t smem = u_bytes + (size_t)best_w * ppw * per_point;
  const long nk = (long)dims[0] * dims[1] * dims[2], per_block = (long)best_w * ppw;
  if (nk > INT_MAX) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH: k mesh too large");
  // frequency ranges of fewer than 2^31 units per launch (32-bit unit indices)
  const int per_launch = (int)std::max(1L, (long)INT_MAX / nk);
  for (int m0 = out.mh0; m0 < out.mh1; m0 += per_launch) {
    PairOut part = out;
    part.mh0 = m0;
    part.mh1 = std::min(out.mh1, m0 + per_launch);
    part.pos = out.pos + (long)(m0 - out.mh0) * out.row;
    part.neg = out.neg ? out.neg + (long)(m0 - out.mh0) * out.neg_step : nullptr;
    const long units = (long)(part.mh1 - part.mh0) * nk;
    long blocks = (units + per_block - 1) / per_block;
    blocks = std::max(1L, std::min(blocks, (long)num_sms() * (best_total / best_w) * 8));
    kern<<<(unsigned)blocks, 32 * best_w, smem, stream>>>(nw, dims[0], dims[1], dims[2], nb, chi0, U, part, status);
    TPRF_KERNEL_LAUNCHED("rpa_pair_kernel");
  }
  return TPRF_OK;
}

template <int G>
int launch_pair_g(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, PairOut chi,
                  cudaStream_t stream, unsigned *status) {
  const bool fp64 = arith_mode() == kArithFP64;
  if (nb == 3)
    return fp64 ? launch_pair_as<double2, G, 3>(nw, dims, nb, chi0, U, chi, stream, status)
                : launch_pair_as<cdf, G, 3>(nw, dims, nb, chi0, U, chi, stream, status);
  if (nb == 5 && G >= 16)
    return fp64 ? launch_pair_as<double2, G, 5>(nw, dims, nb, chi0, U, chi, stream, status)
                : launch_pair_as<cdf, G, 5>(nw, dims, nb, chi0, U, chi, stream, status);
  return fp64 ? launch_pair_as<double2, G, 0>(nw, dims, nb, chi0, U, chi, stream, status)
              : launch_pair_as<cdf, G, 0>(nw, dims, nb, chi0, U, chi, stream, status);
}

int launch_rpa_warp(long n_points, int nb, const double2 *chi0, const double2 *U, double2 *chi, cudaStream_t stream,
                    unsigned *status) {
  auto launch = [&](int lanes, long n) -> int {
    switch (lanes) {
      case 8: return launch_g<8>(n, nb, chi0, U, chi, stream, status);
      case 9: return launch_g<9>(n, nb, chi0, U, chi, stream, status);
      case 16: return launch_g<16>(n, nb, chi0, U, chi, stream, status);
      default: return launch_g<32>(n, nb, chi0, U, chi, stream, status);
    }
  };
  // candidates: the group sizes whose per-warp tiles fit one CTA (as launch_as sizes them)
  const int N = nb * nb;
  const size_t u_bytes = sparse_u_bytes(N);
  std::vector<int> cands;
  // 9 lanes (three groups per warp) own two of the 18 columns of a 9 x 9 system each
  for (int g : {8, 9, 16, 32})
    if ((g != 9 || N == 9) && u_bytes + (size_t)(32 / g) * group_stride(N, g) * 16 <= (size_t)max_smem_optin())
      cands.push_back(g);
  int lanes = rpa_group_lanes(nb);
  const long n_tune = std::min(n_points, (long)num_sms() * 2048);
  if ((const void *)chi0 != (const void *)chi) {
    int st = tune_pick(tune_key("rpa_group", {nb}), cands, lanes, stream, [&](int v) { return launch(v, n_tune); },
                       &lanes);
    if (st) return st;
  }
  return launch(lanes, n_points);
}

// The RPA on a bosonic (w, q) mesh (2 nw - 1 frequencies, k mesh dims) with
// conjugate pairs solved once (rpa_pair_kernel); lanes per point as the point
// form uses (the autotuner's rpa_group wisdom, else the heuristic).
int launch_rpa_warp_pairs(int nw, const int dims[3], int nb, const double2 *chi0, const double2 *U, PairOut out,
                          cudaStream_t stream, unsigned *status) {
  const int N = nb * nb;
  const size_t u_bytes = sparse_u_bytes(N);
  std::vector<int> cands;
  for (int g : {8, 9, 16, 32})
    if ((g != 9 || N == 9) && u_bytes + (size_t)(32 / g) * group_stride(N, g) * 16 <= (size_t)max_smem_optin() - 64)
      cands.push_back(g);
  auto launch = [&](int lanes, PairOut o) -> int {
    switch (lanes) {
      case 8: return launch_pair_g<8>(nw, dims, nb, chi0, U, o, stream, status);
      case 9: return launch_pair_g<9>(nw, dims, nb, chi0, U, o, stream, status);
      case 16: return launch_pair_g<16>(nw, dims, nb, chi0, U, o, stream, status);
      default: return launch_pair_g<32>(nw, dims, nb, chi0, U, o, stream, status);
    }
  };
  int lanes = rpa_group_lanes(nb);
  int st;
  if ((const void *)chi0 != (const void *)(out.pos - (long)(nw - 1 - out.mh0) * out.row)) {
    // a trial is the whole call (it writes what the call writes): trials on the
    // first frequencies ranked the lane counts wrongly (on the 32^3 cubic
    // workload 16 lanes won a 65536-unit and a 524288-unit trial, yet on the full
    // call 9 lanes take 28.9 ms, 16 lanes 29.4 and 8 lanes 30.0)
    st = tune_pick(tune_key("rpa_group", {nb}), cands, lanes, stream, [&](int v) { return launch(v, out); }, &lanes);
  } else {
    st = tune_lookup(tune_key("rpa_group", {nb}), cands, lanes, &lanes);
  }
  if (st) return st;
  return launch(lanes, out);
}

int launch_rpa_adjoint_warp(long n_points, int nb, const double2 *chi0, const double2 *U, const double2 *chi,
                            const double2 *chig, double2 *chi0g, double2 *Ug, cudaStream_t stream, unsigned *status) {
  const int N = nb * nb;
  const size_t u_bytes =
      ((size_t)N * N * (sizeof(double2) + 2 * sizeof(int)) + (N + 1) * sizeof(int) + 15) & ~(size_t)15;
  const size_t per_warp = (size_t)5 * N * N * sizeof(double2);
  const size_t limit = (size_t)max_smem_optin();
  if (u_bytes + per_warp > limit) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_adjoint: nb too large");
  TPRF_CUDA(cudaFuncSetAttribute(rpa_adjoint_warp_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)limit));
  int best_w = 1, best_total = 0;
  for (int w = 1; w <= 16; ++w) {
    const size_t smem = u_bytes + (size_t)w * per_warp;
    if (smem > limit) break;
    int per_sm = 0;
    TPRF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, rpa_adjoint_warp_kernel, 32 * w, smem));
    if (per_sm * w >= best_total) {
      best_total = per_sm * w;
      best_w = w;
    }
  }
  if (best_total == 0) return set_error(TPRF_ERR_INVALID_ARGUMENT, "solve_rpa_PH_adjoint: nb too large");
  const size_t smem = u_bytes + (size_t)best_w * per_warp;
  long blocks = (n_points + best_w - 1) / best_w;
  blocks = std::max(1L, std::min(blocks, (long)num_sms() * (best_total / best_w)));
  rpa_adjoint_warp_kernel<<<(unsigned)blocks, 32 * best_w, smem, stream>>>(n_points, nb, chi0, U, chi, chig, chi0g,
                                                                          Ug, status);
  TPRF_KERNEL_LAUNCHED("rpa_adjoint_warp_kernel");
  return TPRF_OK;
}

int launch_screened_w(long n_points, long nk, int nb, bool swap, bool v_per_point, const double2 *PI, const double2 *V,
                      double2 *W, cudaStream_t stream, unsigned *status) {
  const int N = nb * nb;
  const size_t per_warp = (size_t)4 * N * N * sizeof(double2);
  const size_t limit = (size_t)max_smem_optin();
  if (per_warp > limit) return set_error(TPRF_ERR_INVALID_ARGUMENT, "dynamical_screened_interaction_W: nb too large");
  const int warps = (int)std::max<size_t>(1, std::min<size_t>(8, limit / per_warp));
  const size_t smem = (size_t)warps * per_warp;
  TPRF_CUDA(cudaFuncSetAttribute(screened_w_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  long blocks = (n_points + warps - 1) / warps;
  blocks = std::max(1L, std::min(blocks, (long)num_sms() * 16));
  screened_w_kernel<<<(unsigned)blocks, 32 * warps, smem, stream>>>(n_points, nk, nb, swap ? 1 : 0,
                                                                     v_per_point ? 1 : 0, PI, V, W, status);
  TPRF_KERNEL_LAUNCHED("screened_w_kernel");
  return TPRF_OK;
}

}  // namespace tprf
