// Transposed BSR SpMV that allocates no device memory.
//
// fv_bsr_spmv_f64(..., transpose = 1) builds a transpose map of the block pattern and allocates
// device memory for it on every call.  Callers that cannot allocate device memory while they
// run -- an FFI custom call inside a framework whose allocator owns all device memory (an XLA
// custom call, say), or an embedded solver that forbids allocation after start-up -- use
// fv_bsr_spmv_t_f64_noalloc instead.  It builds the same transpose map on
// the GPU inside one fixed-size scratch array declared below, which every GPU that loads this
// library holds until the process exits.
#include <mutex>

#include "internal.cuh"

// Scratch capacity in ints: the transpose map needs 2 * n_block_rows + 1 + 2 * nnzb of them, plus
// one status word.
#define FV_NOALLOC_SCRATCH_INTS (4 * 1024 * 1024)  // 16 MiB

static __device__ __align__(256) int g_noalloc_scratch[FV_NOALLOC_SCRATCH_INTS];

namespace {

constexpr int kMaxDevices = 64;
int* g_scratch_addr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mutex;

// Device address of the scratch array on the current device.  The symbol lookup runs once per
// device (with that device current); later calls reuse the cached address.
int scratch_address(int** out) {
  int dev = 0;
  FV_CUDA_TRY(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) {
    fv_set_error("fv_bsr_spmv_t_f64_noalloc: device ordinal %d out of range", dev);
    return FV_ERR_ARG;
  }
  std::lock_guard<std::mutex> lock(g_scratch_mutex);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) {
      fv_set_error("fv_bsr_spmv_t_f64_noalloc: cudaGetSymbolAddress failed: %s",
                   cudaGetErrorString(e));
      return FV_ERR_CUDA;
    }
    g_scratch_addr[dev] = (int*)p;
  }
  *out = g_scratch_addr[dev];
  return FV_OK;
}

__global__ void k_na_zero(long n, int* a) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = 0;
}

// cnt[j + 1] = number of stored blocks in block column j
// (column indices outside [0, nbr) are skipped: they cannot address the scratch array)
__global__ void k_na_count(int nbr, const int* ptr, const int* idx, int* cnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbr) return;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    const int j = idx[q];
    if (j >= 0 && j < nbr) atomicAdd(&cnt[j + 1], 1);
  }
}

// In-place inclusive scan of a[0..n) by one block: each thread scans a contiguous chunk, the
// chunk totals are scanned in shared memory, then each chunk adds its offset.  Deterministic.
__global__ void k_na_scan(int n, int* a) {
  __shared__ int tot[1024];
  const int t = threadIdx.x, nt = blockDim.x;
  const int chunk = (n + nt - 1) / nt;
  const int b = min(n, t * chunk), e = min(n, b + chunk);
  int s = 0;
  for (int i = b; i < e; ++i) {
    s += a[i];
    a[i] = s;
  }
  tot[t] = s;
  __syncthreads();
  if (t == 0)
    for (int k = 1; k < nt; ++k) tot[k] += tot[k - 1];
  __syncthreads();
  const int off = t > 0 ? tot[t - 1] : 0;
  for (int i = b; i < e; ++i) a[i] += off;
}

// Place every block (i, j) in column j's segment (arbitrary order within the segment).  Writes
// are bounded by the stated nnzb, so a pattern larger than declared cannot leave the array.
__global__ void k_na_fill(int nbr, long nnzb, const int* ptr, const int* idx, const int* tptr,
                          int* cursor, int* tidx, int* tblk) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nbr) return;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    const int j = idx[q];
    if (j < 0 || j >= nbr) continue;
    const long pos = (long)tptr[j] + atomicAdd(&cursor[j], 1);
    if (pos < nnzb) {
      tidx[pos] = i;
      tblk[pos] = q;
    }
  }
}

// Sort each column segment by row, so the products are summed in ascending row order (the order
// of the host-built map of fv_bsr_spmv_f64) whatever order the fill produced.
__global__ void k_na_sort(int nbc, long nnzb, const int* tptr, int* tidx, int* tblk) {
  int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nbc) return;
  const long end = min((long)tptr[j + 1], nnzb);
  for (long p = tptr[j] + 1; p < end; ++p) {
    const int r = tidx[p], q = tblk[p];
    long k = p - 1;
    while (k >= tptr[j] && tidx[k] > r) {
      tidx[k + 1] = tidx[k];
      tblk[k + 1] = tblk[k];
      --k;
    }
    tidx[k + 1] = r;
    tblk[k + 1] = q;
  }
}

// Status word: 1 when the pattern does not hold exactly nnzb in-range blocks (nnzb differs from
// indptr[n], or some column index lies outside [0, n)); the gather then writes NaN everywhere.
__global__ void k_na_check(int n, long nnzb, const int* ptr, const int* tptr, int* status) {
  *status = ((long)ptr[n] != nnzb || (long)tptr[n] != nnzb) ? 1 : 0;
}

__global__ void k_na_gather(int nbc, long nnzb, int b, const int* tptr, const int* tidx,
                            const int* tblk, const int* status, const double* val,
                            const double* x, double* y) {
  long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (long)nbc * b) return;
  if (*status) {
    y[r] = __longlong_as_double(0x7ff8000000000000LL);  // quiet NaN: the pattern was inconsistent
    return;
  }
  const int j = (int)(r / b), a = (int)(r % b);
  const long bb = (long)b * b;
  double acc = 0.0;
  const long end = min((long)tptr[j + 1], nnzb);
  for (long q = tptr[j]; q < end; ++q) {
    const double* blk = val + (long)tblk[q] * bb;
    const double* xs = x + (long)tidx[q] * b;
    for (int c = 0; c < b; ++c) acc += blk[(long)c * b + a] * xs[c];
  }
  y[r] = acc;
}

}  // namespace

extern "C" int fv_bsr_spmv_t_f64_noalloc(int n_block_rows, long nnzb, int b, const int* indptr,
                                         const int* indices, const double* values, const double* x,
                                         double* y, void* stream) {
  if (n_block_rows <= 0 || nnzb < 0 || b <= 0 || !indptr || !indices || !values || !x || !y) {
    fv_set_error("fv_bsr_spmv_t_f64_noalloc: bad arguments");
    return FV_ERR_ARG;
  }
  const long need = 2L * n_block_rows + 1 + 2 * nnzb + 1;
  if (need > FV_NOALLOC_SCRATCH_INTS) {
    fv_set_error(
        "fv_bsr_spmv_t_f64_noalloc: the pattern needs %ld scratch ints (2 * n_block_rows + 2 + "
        "2 * nnzb) but the fixed scratch array holds %d; use fv_bsr_spmv_f64 with transpose = 1",
        need, FV_NOALLOC_SCRATCH_INTS);
    return FV_ERR_ARG;
  }
  int* base = nullptr;
  int rc = scratch_address(&base);
  if (rc != FV_OK) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = n_block_rows;
  int* tptr = base;             // n + 1: column counts, then column starts
  int* cursor = tptr + n + 1;   // n
  int* tidx = cursor + n;       // nnzb
  int* tblk = tidx + nnzb;      // nnzb
  int* status = tblk + nnzb;    // 1
  // counts and cursors must start at zero; the map entries are fully overwritten
  k_na_zero<<<fv_blocks(2L * n + 1, 256), 256, 0, s>>>(2L * n + 1, tptr);
  k_na_count<<<fv_blocks(n, 256), 256, 0, s>>>(n, indptr, indices, tptr);
  k_na_scan<<<1, 1024, 0, s>>>(n + 1, tptr);
  k_na_fill<<<fv_blocks(n, 256), 256, 0, s>>>(n, nnzb, indptr, indices, tptr, cursor, tidx, tblk);
  k_na_check<<<1, 1, 0, s>>>(n, nnzb, indptr, tptr, status);
  k_na_sort<<<fv_blocks(n, 256), 256, 0, s>>>(n, nnzb, tptr, tidx, tblk);
  k_na_gather<<<fv_blocks((long)n * b, 256), 256, 0, s>>>(n, nnzb, b, tptr, tidx, tblk, status,
                                                         values, x, y);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}
