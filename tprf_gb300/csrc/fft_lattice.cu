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
// (target index fastest, as in HBM). One CTA loads a tile of columns
// (consecutive inner indices, and several outer slices when inner is short)
// into shared memory with coalesced row reads, runs a mixed-radix Stockham
// FFT on all columns at once and writes the tile back. One pass per mesh
// dimension with n > 1; later passes run in place.
#include <algorithm>

#include "common.cuh"

namespace tprf {
namespace {

template <bool FWD>
__global__ void __launch_bounds__(256) lattice_axis_kernel(const double2 *in, double2 *out, long outer, long inner,
                                                           int oc, int ic, FftDesc d, double scale) {
  extern __shared__ double2 smem[];
  const int n = d.n;
  const int ncol = oc * ic;
  double2 *a = smem;
  double2 *b = smem + (size_t)n * ncol;
  const long n_ichunk = (inner + ic - 1) / ic;
  const long o0 = (blockIdx.x / n_ichunk) * oc;
  const long i0 = (blockIdx.x % n_ichunk) * ic;
  const int tid = threadIdx.x, nthr = blockDim.x;
  const int tile = n * ncol;
  for (int w = tid; w < tile; w += nthr) {
    const int il = w % ic;
    const int row = (w / ic) % n;
    const int ol = w / (ic * n);
    const long o = o0 + ol, i = i0 + il;
    double2 v = make_double2(0.0, 0.0);
    if (o < outer && i < inner) v = in[(o * n + row) * inner + i];
    a[row * ncol + ol * ic + il] = v;
  }
  double2 *r = fft_smem<FWD>(a, b, d, ncol);
  for (int w = tid; w < tile; w += nthr) {
    const int il = w % ic;
    const int row = (w / ic) % n;
    const int ol = w / (ic * n);
    const long o = o0 + ol, i = i0 + il;
    if (o < outer && i < inner) out[(o * n + row) * inner + i] = cscale(r[row * ncol + ol * ic + il], scale);
  }
}

template <bool FWD>
int launch_axis(const double2 *in, double2 *out, long outer, int n, long inner, double scale, cudaStream_t stream) {
  FftDesc d;
  int st = get_fft(n, &d);
  if (st) return st;
  // Tile of ~64 columns, limited by shared memory (two buffers of n x ncol).
  const int budget = std::min(max_smem_optin(), 200 * 1024);
  int max_cols = budget / (2 * n * (int)sizeof(double2));
  if (max_cols < 1) return set_error(TPRF_ERR_UNSUPPORTED_SIZE, "lattice FFT: mesh dimension too long for one CTA");
  int want = std::min(64, max_cols);
  int ic, oc;
  if (inner >= want) {
    ic = want;
    oc = 1;
  } else {
    ic = (int)inner;
    oc = std::max(1, want / ic);
    oc = (int)std::min<long>(oc, outer);
  }
  const size_t smem = 2ull * n * oc * ic * sizeof(double2);
  const long n_ichunk = (inner + ic - 1) / ic;
  const long n_ochunk = (outer + oc - 1) / oc;
  const long blocks = n_ichunk * n_ochunk;
  if (blocks > 0x7fffffffL) return set_error(TPRF_ERR_INVALID_ARGUMENT, "lattice FFT: too many tiles");
  TPRF_CUDA(cudaFuncSetAttribute(lattice_axis_kernel<FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  lattice_axis_kernel<FWD><<<(unsigned)blocks, 256, smem, stream>>>(in, out, outer, inner, oc, ic, d, scale);
  TPRF_LAUNCH_CHECK("lattice_axis_kernel");
  return TPRF_OK;
}

}  // namespace

// Transform over the 3 mesh dims of [n_w, dims..., n_target]; in == out allowed.
int launch_lattice_fft(bool forward, long n_w, const int dims[3], long n_target, const double2 *in, double2 *out,
                       cudaStream_t stream) {
  const long nk = (long)dims[0] * dims[1] * dims[2];
  int last = -1;
  for (int ax = 0; ax < 3; ++ax)
    if (dims[ax] > 1) last = ax;
  if (last < 0) {  // a single k point: the transform is the identity
    if (in != out) TPRF_CUDA(cudaMemcpyAsync(out, in, n_w * n_target * sizeof(double2), cudaMemcpyDeviceToDevice, stream));
    return TPRF_OK;
  }
  const double scale_last = forward ? 1.0 / (double)nk : 1.0;
  const double2 *src = in;
  // fastest-varying mesh dimension first: its pass has the longest contiguous rows
  for (int ax = 2; ax >= 0; --ax) {
    const int n = dims[ax];
    if (n <= 1) continue;
    long outer = n_w, inner = n_target;
    for (int a2 = 0; a2 < ax; ++a2) outer *= dims[a2];
    for (int a2 = ax + 1; a2 < 3; ++a2) inner *= dims[a2];
    // scale once, on the last pass issued (the slowest dimension with n > 1)
    int first_nontrivial = 0;
    while (dims[first_nontrivial] <= 1) ++first_nontrivial;
    const double scale = (ax == first_nontrivial) ? scale_last : 1.0;
    int st = forward ? launch_axis<true>(src, out, outer, n, inner, scale, stream)
                     : launch_axis<false>(src, out, outer, n, inner, scale, stream);
    if (st) return st;
    src = out;
  }
  (void)last;
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
