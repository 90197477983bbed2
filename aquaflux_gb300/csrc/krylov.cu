// Flexible GMRES(m) building blocks on the device, fp64, deterministic.
//
// The reference's linear solve is lineax GMRES (aquaflux/solve/linear.py:199-298, restart and
// tolerances from linear.py:40-42 and implicit.py:50): right-preconditioned, restarted, with the
// residual estimate of the rotated least-squares problem as the stopping test.  Here one Arnoldi
// step is four launches and never returns to the host:
//   k_proj         h1 = V[0..k)^T w                                  (CGS, first pass)
//   k_upd<true>    w -= V h1;  h2 = V[0..k)^T w                      (CGS, second pass)
//   k_upd_norm     w -= V h2;  ||w||; the last block writes the Hessenberg column h1 + h2,
//                  ||w||, applies the previous Givens rotations, forms the new one, and updates
//                  the rotated right-hand side g (residual estimate |g[j+1]|)
//   k_scale        V[j+1] = w / ||w||
// Every reduction is a fixed grid of kRedBlocks blocks over a grid-stride loop, block partials
// summed in a fixed order by the last block to finish (a ticket counter), so results are bitwise
// identical run to run.  Up to kChunk basis vectors are handled per launch; a longer basis is
// processed chunk by chunk with the update and the projection in separate passes.
#include <algorithm>
#include <cmath>

#include "internal.cuh"

namespace {

constexpr int kThreads = 256;          // 8 warps
constexpr int kWarps = kThreads / 32;
constexpr int kRedBlocks = 4 * 152;     // fixed, so the summation order never changes
constexpr int kChunk = 32;              // basis vectors per launch
constexpr int kSlots = kChunk / kWarps; // projections per warp

// The projection kernels walk tiles of kThreads entries (grid-stride over tiles): the tile of w
// goes to shared memory, then warp u accumulates the dot products of the basis vectors
// v = u, u + kWarps, ... with it, each lane over 8 coalesced entries of the tile.  Registers stay
// few (kSlots accumulators), so occupancy is high; every partial sum runs in a fixed order.
__device__ __forceinline__ void tile_project(long n, long base, int k, const double* __restrict__ V,
                                             const double* ws, double (&acc)[kSlots]) {
  const int lane = threadIdx.x & 31, u = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < kSlots; ++t) {
    const int v = u + t * kWarps;
    if (v >= k) break;
    const double* row = V + (long)v * n + base;
    double a = acc[t];
#pragma unroll
    for (int e = 0; e < kThreads / 32; ++e) {
      const int i = lane + 32 * e;
      if (base + i < n) a = fma(row[i], ws[i], a);
    }
    acc[t] = a;
  }
}

// Write this block's partials: part[blockIdx.x * k + v] = the block's sum for vector v.
__device__ __forceinline__ void write_partials(const double (&acc)[kSlots], int k, double* part) {
  __shared__ double sh[kChunk];
  const int lane = threadIdx.x & 31, u = threadIdx.x >> 5;
#pragma unroll
  for (int t = 0; t < kSlots; ++t) {
    const int v = u + t * kWarps;
    double x = acc[t];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    if (lane == 0 && v < k) sh[v] = x;
  }
  __syncthreads();
  if (threadIdx.x < k) part[(long)blockIdx.x * k + threadIdx.x] = sh[threadIdx.x];
}

// After every block wrote its k partials: the last block to finish sums them in a fixed order
// (warp u sums vectors u, u + kWarps, ...: lane l over blocks l, l + 32, ..., then a fixed
// shuffle tree) into res[0..k) and returns true (in every thread of that block).
__device__ __forceinline__ bool last_block_sum(const double* part, int k, unsigned* ticket,
                                               double* res) {
  __shared__ bool last;
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  const int lane = threadIdx.x & 31, u = threadIdx.x >> 5;
  const volatile double* vp = part;
  for (int v = u; v < k; v += kWarps) {
    double s = 0.0;
    for (int b = lane; b < (int)gridDim.x; b += 32) s += vp[(long)b * k + v];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) res[v] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) *ticket = 0u;  // ready for the next reduction on this workspace
  return true;
}

// h[0..k) = V[0..k)^T w  (V rows of length n at stride n).
__global__ void __launch_bounds__(kThreads) k_proj(long n, int k, const double* __restrict__ V,
                                                   const double* __restrict__ w, double* part,
                                                   unsigned* ticket, double* h) {
  __shared__ double ws[kThreads];
  double acc[kSlots];
#pragma unroll
  for (int t = 0; t < kSlots; ++t) acc[t] = 0.0;
  for (long base = (long)blockIdx.x * kThreads; base < n; base += (long)gridDim.x * kThreads) {
    const long i = base + threadIdx.x;
    __syncthreads();
    ws[threadIdx.x] = i < n ? w[i] : 0.0;
    __syncthreads();
    tile_project(n, base, k, V, ws, acc);
  }
  write_partials(acc, k, part);
  last_block_sum(part, k, ticket, h);
}

// w -= V[0..k)^T-combination with coefficients c; then (PROJ) h = V[0..k)^T w of the new w, the
// tile's basis entries read a second time from cache.
template <bool PROJ>
__global__ void __launch_bounds__(kThreads) k_upd(long n, int k, const double* __restrict__ V,
                                                  const double* __restrict__ c,
                                                  double* __restrict__ w, double* part,
                                                  unsigned* ticket, double* h) {
  __shared__ double cs[kChunk];
  __shared__ double ws[kThreads];
  if (threadIdx.x < k) cs[threadIdx.x] = c[threadIdx.x];
  double acc[kSlots];
#pragma unroll
  for (int t = 0; t < kSlots; ++t) acc[t] = 0.0;
  for (long base = (long)blockIdx.x * kThreads; base < n; base += (long)gridDim.x * kThreads) {
    const long i = base + threadIdx.x;
    __syncthreads();
    double wi = 0.0;
    if (i < n) {
      wi = w[i];
#pragma unroll 8
      for (int v = 0; v < k; ++v) wi = fma(-cs[v], V[(long)v * n + i], wi);
      w[i] = wi;
    }
    if (PROJ) {
      ws[threadIdx.x] = wi;
      __syncthreads();
      tile_project(n, base, k, V, ws, acc);
    }
  }
  if (!PROJ) return;
  write_partials(acc, k, part);
  last_block_sum(part, k, ticket, h);
}

struct Hess {
  int m;         // restart length: H is (m + 1) x m, column-major
  double* H;
  double* cs;
  double* sn;
  double* g;     // (m + 1) rotated right-hand side
  double* est;   // (2) |g[j + 1]| and h[j + 1, j] of the last column
  double* inv;   // (1) 1 / ||w|| (1 on a breakdown), the normalisation of V[j + 1]
};

// Column j of the Hessenberg matrix from the two CGS projections and ||w||, then the Givens
// reduction (one thread; j < m).
__device__ void finish_column(Hess hs, int j, const double* h1, const double* h2, double nrm) {
  double* col = hs.H + (long)j * (hs.m + 1);
  for (int i = 0; i <= j; ++i) col[i] = h1[i] + h2[i];
  col[j + 1] = nrm;
  for (int i = 0; i < j; ++i) {  // the previous rotations
    const double t = hs.cs[i] * col[i] + hs.sn[i] * col[i + 1];
    col[i + 1] = -hs.sn[i] * col[i] + hs.cs[i] * col[i + 1];
    col[i] = t;
  }
  const double den = hypot(col[j], col[j + 1]);
  double c = 1.0, s = 0.0;
  if (den != 0.0) {
    c = col[j] / den;
    s = col[j + 1] / den;
  }
  hs.cs[j] = c;
  hs.sn[j] = s;
  col[j] = c * col[j] + s * col[j + 1];
  col[j + 1] = 0.0;
  const double gj = hs.g[j];
  hs.g[j + 1] = -s * gj;
  hs.g[j] = c * gj;
  hs.est[0] = fabs(hs.g[j + 1]);
  hs.est[1] = nrm;
  hs.inv[0] = nrm > 0.0 ? 1.0 / nrm : 1.0;
}

// What the last block of k_upd_norm does with ||w||.
enum NormMode { NM_COLUMN = 0, NM_START = 1, NM_ONLY = 2 };

// w -= V[0..k)^T-combination with coefficients c (when k > 0); ||w||^2 reduced; the last block
// then finishes column j (NM_COLUMN), starts a cycle: g = (||w||, 0, ...) (NM_START), or only
// stores ||w|| in *nrm_out (NM_ONLY).
__global__ void __launch_bounds__(kThreads) k_upd_norm(long n, int k, const double* __restrict__ V,
                                                       const double* __restrict__ c,
                                                       double* __restrict__ w, double* part,
                                                       unsigned* ticket, double* red, Hess hs,
                                                       int mode, int j, const double* h1,
                                                       const double* h2, double* nrm_out) {
  __shared__ double cs[kChunk];
  if (threadIdx.x < k) cs[threadIdx.x] = c[threadIdx.x];
  __syncthreads();
  double acc = 0.0;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    double wi = w[i];
#pragma unroll 8
    for (int v = 0; v < k; ++v) wi = fma(-cs[v], V[(long)v * n + i], wi);
    if (k > 0) w[i] = wi;
    acc = fma(wi, wi, acc);
  }
  // block sum in a fixed order: warp shuffles, then the warp totals by thread 0
  __shared__ double sh[kWarps];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int u = 0; u < kWarps; ++u) t += sh[u];
    part[blockIdx.x] = t;
  }
  if (last_block_sum(part, 1, ticket, red) && threadIdx.x == 0) {
    const double nrm = sqrt(red[0]);
    if (mode == NM_COLUMN) {
      finish_column(hs, j, h1, h2, nrm);
    } else if (mode == NM_START) {
      for (int i = 0; i <= hs.m; ++i) hs.g[i] = i == 0 ? nrm : 0.0;
      hs.est[0] = nrm;
      hs.est[1] = nrm;
      hs.inv[0] = nrm > 0.0 ? 1.0 / nrm : 1.0;
    } else {
      *nrm_out = nrm;
    }
  }
}

// out = w * inv[0]
__global__ void k_scale(long n, const double* __restrict__ w, const double* __restrict__ inv,
                        double* __restrict__ out) {
  const double s = *inv;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    out[i] = w[i] * s;
}

// y = H[0..k, 0..k)^-1 g[0..k) by back substitution (one thread).
__global__ void k_backsolve(Hess hs, int k, double* y) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  for (int i = k - 1; i >= 0; --i) {
    double t = hs.g[i];
    for (int l = i + 1; l < k; ++l) t -= hs.H[(long)l * (hs.m + 1) + i] * y[l];
    y[i] = t / hs.H[(long)i * (hs.m + 1) + i];
  }
}

// x += Z[0..k)^T y  (k <= kChunk per launch; chunks applied in order)
__global__ void k_combine(long n, int k, const double* __restrict__ Z, const double* __restrict__ y,
                          double* __restrict__ x) {
  __shared__ double ys[kChunk];
  if (threadIdx.x < k) ys[threadIdx.x] = y[threadIdx.x];
  __syncthreads();
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
    double xi = x[i];
#pragma unroll 8
    for (int v = 0; v < k; ++v) xi = fma(ys[v], Z[(long)v * n + i], xi);
    x[i] = xi;
  }
}

}  // namespace

struct FvKrylov {
  int m = 0;
  double* buf = nullptr;  // H, cs, sn, g, est, inv, h1, h2, y, red, partials
  unsigned* ticket = nullptr;
  Hess hs{};
  double *h1 = nullptr, *h2 = nullptr, *y = nullptr, *red = nullptr, *part = nullptr;
};

extern "C" int fv_krylov_create(int m, FvKrylov** out) {
  if (!out || m <= 0 || m > 4096) {
    fv_set_error("fv_krylov_create: restart length must be in [1, 4096]");
    return FV_ERR_ARG;
  }
  FvKrylov* kr = new FvKrylov();
  kr->m = m;
  const long nH = (long)(m + 1) * m;
  const long total = nH + m + m + (m + 1) + 2 + 1 + (m + 1) + (m + 1) + m + 1 +
                     (long)kRedBlocks * kChunk;
  cudaError_t e = cudaMalloc(&kr->buf, sizeof(double) * total);
  if (e == cudaSuccess) e = cudaMalloc(&kr->ticket, sizeof(unsigned));
  if (e == cudaSuccess) e = cudaMemset(kr->ticket, 0, sizeof(unsigned));
  if (e != cudaSuccess) {
    cudaFree(kr->buf);
    cudaFree(kr->ticket);
    delete kr;
    fv_set_error("fv_krylov_create: %s", cudaGetErrorString(e));
    return FV_ERR_CUDA;
  }
  double* p = kr->buf;
  kr->hs.m = m;
  kr->hs.H = p; p += nH;
  kr->hs.cs = p; p += m;
  kr->hs.sn = p; p += m;
  kr->hs.g = p; p += m + 1;
  kr->hs.est = p; p += 2;
  kr->hs.inv = p; p += 1;
  kr->h1 = p; p += m + 1;
  kr->h2 = p; p += m + 1;
  kr->y = p; p += m;
  kr->red = p; p += 1;
  kr->part = p;
  *out = kr;
  return FV_OK;
}

extern "C" int fv_krylov_destroy(FvKrylov* kr) {
  if (!kr) return FV_OK;
  cudaFree(kr->buf);
  cudaFree(kr->ticket);
  delete kr;
  return FV_OK;
}

extern "C" int fv_krylov_start(FvKrylov* kr, long n, const double* r, double* v0, double* est,
                               void* stream) {
  if (!kr || n <= 0 || !r || !v0) {
    fv_set_error("fv_krylov_start: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  k_upd_norm<<<kRedBlocks, kThreads, 0, s>>>(n, 0, nullptr, nullptr, const_cast<double*>(r),
                                              kr->part, kr->ticket, kr->red, kr->hs, NM_START, -1,
                                              nullptr, nullptr, nullptr);
  k_scale<<<kRedBlocks, kThreads, 0, s>>>(n, r, kr->hs.inv, v0);
  if (est) FV_CUDA_TRY(cudaMemcpyAsync(est, kr->hs.est, 2 * sizeof(double), cudaMemcpyDefault, s));
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_krylov_arnoldi(FvKrylov* kr, int j, long n, double* V, double* w, double* est,
                                 void* stream) {
  if (!kr || j < 0 || j >= kr->m || n <= 0 || !V || !w) {
    fv_set_error("fv_krylov_arnoldi: bad arguments (0 <= j < m)");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int k = j + 1;  // basis vectors V[0..k)
  if (k <= kChunk) {
    k_proj<<<kRedBlocks, kThreads, 0, s>>>(n, k, V, w, kr->part, kr->ticket, kr->h1);
    k_upd<true><<<kRedBlocks, kThreads, 0, s>>>(n, k, V, kr->h1, w, kr->part, kr->ticket, kr->h2);
    k_upd_norm<<<kRedBlocks, kThreads, 0, s>>>(n, k, V, kr->h2, w, kr->part, kr->ticket, kr->red,
                                                kr->hs, NM_COLUMN, j, kr->h1, kr->h2, nullptr);
  } else {
    // chunked CGS2: project all chunks, update by all chunks, twice; then the norm
    for (int pass = 0; pass < 2; ++pass) {
      double* h = pass == 0 ? kr->h1 : kr->h2;
      for (int c0 = 0; c0 < k; c0 += kChunk)
        k_proj<<<kRedBlocks, kThreads, 0, s>>>(n, std::min(kChunk, k - c0), V + (long)c0 * n, w,
                                               kr->part, kr->ticket, h + c0);
      for (int c0 = 0; c0 < k; c0 += kChunk)
        k_upd<false><<<kRedBlocks, kThreads, 0, s>>>(n, std::min(kChunk, k - c0),
                                                     V + (long)c0 * n, h + c0, w, nullptr,
                                                     nullptr, nullptr);
    }
    k_upd_norm<<<kRedBlocks, kThreads, 0, s>>>(n, 0, nullptr, nullptr, w, kr->part, kr->ticket,
                                                kr->red, kr->hs, NM_COLUMN, j, kr->h1, kr->h2,
                                                nullptr);
  }
  k_scale<<<kRedBlocks, kThreads, 0, s>>>(n, w, kr->hs.inv, V + (long)k * n);
  if (est) FV_CUDA_TRY(cudaMemcpyAsync(est, kr->hs.est, 2 * sizeof(double), cudaMemcpyDefault, s));
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_krylov_update(FvKrylov* kr, int k, long n, const double* Z, double* x,
                                void* stream) {
  if (!kr || k < 0 || k > kr->m || n <= 0 || !Z || !x) {
    fv_set_error("fv_krylov_update: bad arguments (0 <= k <= m)");
    return FV_ERR_ARG;
  }
  if (k == 0) return FV_OK;
  cudaStream_t s = (cudaStream_t)stream;
  k_backsolve<<<1, 32, 0, s>>>(kr->hs, k, kr->y);
  for (int c0 = 0; c0 < k; c0 += kChunk)
    k_combine<<<kRedBlocks, kThreads, 0, s>>>(n, std::min(kChunk, k - c0), Z + (long)c0 * n,
                                              kr->y + c0, x);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_krylov_norm(FvKrylov* kr, long n, const double* x, double* out, void* stream) {
  if (!kr || n <= 0 || !x || !out) {
    fv_set_error("fv_krylov_norm: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  // k = 0: x is only read
  k_upd_norm<<<kRedBlocks, kThreads, 0, s>>>(n, 0, nullptr, nullptr, const_cast<double*>(x),
                                              kr->part, kr->ticket, kr->red, kr->hs, NM_ONLY, -1,
                                              nullptr, nullptr, out);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}
