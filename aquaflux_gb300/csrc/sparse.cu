// Block-sparse (BSR) SpMV, zero-fill ILU(0) and deterministic reductions.
//
// ILU(0) restates aquaflux/solve/_ilu0.pyx (factor :68-121, solve :124-147, solve_transpose
// :150-178) for b x b dense blocks.  On a block-dense pattern, scalar IKJ ILU(0) over the
// block-expanded (cell-major interleaved) ordering is the same elimination as:
//   for each lower block (i, j), ascending j:   L_ij = A_ij U_jj^-1   (U_jj: upper triangle of the
//                                                factored diagonal block of row j)
//                                                A_ik -= L_ij A_jk   for k > j stored in both rows
//   then the in-place unit-lower / upper LU of A_ii and A_ik = L_ii^-1 A_ik for k > i,
// which is what one thread does per block row here.  Rows run in level-set order (a row's level
// is one more than the deepest row it depends on), so the factor and the triangular sweeps
// reproduce the sequential algorithm's dependencies exactly.  With b = 1 this is the reference's
// scalar CSR ILU(0).
#include <algorithm>
#include <cstdio>
#include <type_traits>
#include <memory>
#include <vector>

#include "internal.cuh"

void fv_set_error_index(long i);

namespace {

constexpr int kThreads = 256;

// B contiguous values p[0 .. B) into registers with the widest vector loads the block size allows
// (p is aligned to B values: every block row segment and every cell segment is).
template <int B, class V>
__device__ __forceinline__ void load_seg(const V* __restrict__ p, V (&o)[B]) {
  if constexpr (std::is_same<V, double>::value && B % 2 == 0) {
#pragma unroll
    for (int k = 0; k < B / 2; ++k) {
      const double2 t = reinterpret_cast<const double2*>(p)[k];
      o[2 * k] = t.x;
      o[2 * k + 1] = t.y;
    }
  } else if constexpr (std::is_same<V, float>::value && B % 4 == 0) {
#pragma unroll
    for (int k = 0; k < B / 4; ++k) {
      const float4 t = reinterpret_cast<const float4*>(p)[k];
      o[4 * k] = t.x;
      o[4 * k + 1] = t.y;
      o[4 * k + 2] = t.z;
      o[4 * k + 3] = t.w;
    }
  } else if constexpr (std::is_same<V, float>::value && B % 2 == 0) {
#pragma unroll
    for (int k = 0; k < B / 2; ++k) {
      const float2 t = reinterpret_cast<const float2*>(p)[k];
      o[2 * k] = t.x;
      o[2 * k + 1] = t.y;
    }
  } else {
#pragma unroll
    for (int k = 0; k < B; ++k) o[k] = p[k];
  }
}

// a * b + c with one rounding.
__device__ __forceinline__ float fma_rn(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double fma_rn(double a, double b, double c) { return __fma_rn(a, b, c); }

// Calls fn(std::integral_constant<int, B>) for the runtime block size b in 2 .. 8.
template <class Fn>
void with_block_size(int b, Fn&& fn) {
  switch (b) {
    case 2: fn(std::integral_constant<int, 2>{}); break;
    case 3: fn(std::integral_constant<int, 3>{}); break;
    case 4: fn(std::integral_constant<int, 4>{}); break;
    case 5: fn(std::integral_constant<int, 5>{}); break;
    case 6: fn(std::integral_constant<int, 6>{}); break;
    case 7: fn(std::integral_constant<int, 7>{}); break;
    default: fn(std::integral_constant<int, 8>{}); break;
  }
}


// ------------------------------------------------------------------------------ BSR SpMV
template <class V>
__global__ void k_bsr_spmv(int nbr, int b, const int* __restrict__ ptr, const int* __restrict__ idx,
                           const V* __restrict__ val, const V* __restrict__ x, V* __restrict__ y) {
  // one thread per scalar row: row r = (block row i, component a)
  long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (long)nbr * b) return;
  int i = (int)(r / b), a = (int)(r % b);
  V acc = 0;
  const long bb = (long)b * b;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    const V* blk = val + (long)q * bb + (long)a * b;
    const V* xs = x + (long)idx[q] * b;
    for (int c = 0; c < b; ++c) acc += blk[c] * xs[c];
  }
  y[r] = acc;
}

// The same product with a compile-time block size and vector loads of each row segment (every
// block row segment and x segment starts at a multiple of B values from 16-byte aligned bases).
template <class V, int B>
__global__ void k_bsr_spmv_b(int nbr, const int* __restrict__ ptr, const int* __restrict__ idx,
                             const V* __restrict__ val, const V* __restrict__ x,
                             V* __restrict__ y) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (long)nbr * B) return;
  const int i = (int)(r / B), a = (int)(r % B);
  constexpr long BB = (long)B * B;
  V acc = 0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    V m[B], xs[B];
    load_seg<B>(val + (long)q * BB + (long)a * B, m);
    load_seg<B>(x + (long)idx[q] * B, xs);
#pragma unroll
    for (int c = 0; c < B; ++c) acc += m[c] * xs[c];
  }
  y[r] = acc;
}

// Transposed product through the precomputed transpose map: for block row j of A^T, gather
// blocks (i, j) of A (tptr/tidx list rows i, tblk the block index in A).
template <class V>
__global__ void k_bsr_spmv_t(int nbc, int b, const int* __restrict__ tptr, const int* __restrict__ tidx,
                             const int* __restrict__ tblk, const V* __restrict__ val,
                             const V* __restrict__ x, V* __restrict__ y) {
  long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (long)nbc * b) return;
  int j = (int)(r / b), a = (int)(r % b);
  V acc = 0;
  const long bb = (long)b * b;
  for (int q = tptr[j]; q < tptr[j + 1]; ++q) {
    const V* blk = val + (long)tblk[q] * bb;
    const V* xs = x + (long)tidx[q] * b;
    for (int c = 0; c < b; ++c) acc += blk[(long)c * b + a] * xs[c];
  }
  y[r] = acc;
}

// The same transposed product with a compile-time block size: the same products accumulated in
// the same order (bitwise the runtime-size kernel's result), the loops unrolled.
template <class V, int B>
__global__ void k_bsr_spmv_tb(int nbc, const int* __restrict__ tptr, const int* __restrict__ tidx,
                              const int* __restrict__ tblk, const V* __restrict__ val,
                              const V* __restrict__ x, V* __restrict__ y) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= (long)nbc * B) return;
  const int j = (int)(r / B), a = (int)(r % B);
  constexpr long BB = (long)B * B;
  V acc = 0;
  for (int q = tptr[j]; q < tptr[j + 1]; ++q) {
    const V* blk = val + (long)tblk[q] * BB + a;
    V xs[B];
    load_seg<B>(x + (long)tidx[q] * B, xs);
#pragma unroll
    for (int c = 0; c < B; ++c) acc += blk[(long)c * B] * xs[c];
  }
  y[r] = acc;
}

// y = A^T x through a device transpose map, the compile-time-size kernel for b in 2 .. 8 (x
// 16-byte aligned: its segments are read with vector loads).
template <class V>
void launch_spmv_t(int n, int b, const int* tp, const int* ti, const int* tb, const V* values,
                   const V* x, V* y, cudaStream_t s) {
  const long rows = (long)n * b;
  if (b >= 2 && b <= 8 && (uintptr_t)x % 16 == 0)
    with_block_size(b, [&](auto B) {
      k_bsr_spmv_tb<V, B()><<<fv_blocks(rows, kThreads), kThreads, 0, s>>>(n, tp, ti, tb, values,
                                                                           x, y);
    });
  else
    k_bsr_spmv_t<V><<<fv_blocks(rows, kThreads), kThreads, 0, s>>>(n, b, tp, ti, tb, values, x, y);
}

// tval[q] = val[tblk[q]]^T: the blocks of A in the order of A^T's pattern, each transposed, so
// that row a of block q of A^T is contiguous (the transposed sweeps and products read it with
// the forward kernels' vector loads).
template <class V>
__global__ void k_transpose_blocks(long nnzb, int b, const int* __restrict__ tblk,
                                   const V* __restrict__ val, V* __restrict__ tval) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long bb = (long)b * b;
  if (t >= nnzb * bb) return;
  const long q = t / bb;
  const int e = (int)(t - q * bb), r = e / b, c = e - r * b;
  tval[t] = val[(long)tblk[q] * bb + (long)c * b + r];
}

// Host-built transpose of a BSR pattern (cached per pattern pointer for the SpMV entry points).
struct Transpose {
  std::vector<int> ptr, idx, blk;
};
void build_transpose(int nbr, int nbc, const int* ptr, const int* idx, Transpose* t) {
  t->ptr.assign(nbc + 1, 0);
  for (int i = 0; i < nbr; ++i)
    for (int q = ptr[i]; q < ptr[i + 1]; ++q) t->ptr[idx[q] + 1]++;
  for (int j = 0; j < nbc; ++j) t->ptr[j + 1] += t->ptr[j];
  t->idx.assign(t->ptr[nbc], 0);
  t->blk.assign(t->ptr[nbc], 0);
  std::vector<int> fill(t->ptr.begin(), t->ptr.end() - 1);
  for (int i = 0; i < nbr; ++i)
    for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
      int s = fill[idx[q]]++;
      t->idx[s] = i;
      t->blk[s] = q;
    }
}

// ------------------------------------------------------------------------------ ILU(0)
template <class V>
struct IluView {
  int n, b;
  const int* ptr;
  const int* idx;
  const int* diag;  // block index of the diagonal block of each row
  V* val;
};

__device__ __forceinline__ void note_zero_pivot(unsigned long long* flag, int row, int col) {
  unsigned long long key = ((unsigned long long)(unsigned)row << 32) | (unsigned)col;
  atomicMin(flag, key);
}

// Factor the block rows of one level.  One thread per block row.
template <class V>
__global__ void k_ilu_factor_level(IluView<V> F, const int* rows, int count,
                                   unsigned long long* zero_flag) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t];
  const int b = F.b;
  const long bb = (long)b * b;
  const int rb = F.ptr[i], re = F.ptr[i + 1], di = F.diag[i];
  // lower blocks, ascending column
  for (int q = rb; q < di; ++q) {
    const int j = F.idx[q];
    V* Lij = F.val + (long)q * bb;
    const V* Ujj = F.val + (long)F.diag[j] * bb;
    // L_ij = A_ij U_jj^-1, column by column (scalar columns jb ascending)
    for (int cb = 0; cb < b; ++cb) {
      const V piv = Ujj[(long)cb * b + cb];
      if (piv == V(0)) note_zero_pivot(zero_flag, i * b, j * b + cb);
      for (int a = 0; a < b; ++a) {
        V l = Lij[(long)a * b + cb] / piv;
        Lij[(long)a * b + cb] = l;
        for (int c2 = cb + 1; c2 < b; ++c2) Lij[(long)a * b + c2] -= l * Ujj[(long)cb * b + c2];
      }
    }
    // A_ik -= L_ij A_jk for k > j present in both rows (merge of sorted column lists)
    int p = q + 1;
    for (int s = F.diag[j] + 1; s < F.ptr[j + 1]; ++s) {
      const int k = F.idx[s];
      while (p < re && F.idx[p] < k) ++p;
      if (p >= re) break;
      if (F.idx[p] != k) continue;
      V* Aik = F.val + (long)p * bb;
      const V* Ajk = F.val + (long)s * bb;
      for (int a = 0; a < b; ++a)
        for (int c = 0; c < b; ++c) {
          V acc = Aik[(long)a * b + c];
          for (int m = 0; m < b; ++m) acc -= Lij[(long)a * b + m] * Ajk[(long)m * b + c];
          Aik[(long)a * b + c] = acc;
        }
    }
  }
  // diagonal block: in-place LU (unit lower), and L_ii^-1 applied to the upper blocks
  V* D = F.val + (long)di * bb;
  for (int cb = 0; cb < b; ++cb) {
    const V piv = D[(long)cb * b + cb];
    for (int a = cb + 1; a < b; ++a) {
      if (piv == V(0)) note_zero_pivot(zero_flag, i * b + a, i * b + cb);
      V l = D[(long)a * b + cb] / piv;
      D[(long)a * b + cb] = l;
      for (int c = cb + 1; c < b; ++c) D[(long)a * b + c] -= l * D[(long)cb * b + c];
      for (int q = di + 1; q < re; ++q) {
        V* U = F.val + (long)q * bb;
        for (int c = 0; c < b; ++c) U[(long)a * b + c] -= l * U[(long)cb * b + c];
      }
    }
  }
}

// Forward sweep (L y = r, unit lower) for one level; y holds r on entry.
template <class V>
__global__ void k_ilu_lower(IluView<V> F, const int* rows, int count, V* y) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t], b = F.b;
  const long bb = (long)b * b;
  V acc[8];
  for (int a = 0; a < b; ++a) acc[a] = y[(long)i * b + a];
  for (int q = F.ptr[i]; q < F.diag[i]; ++q) {
    const V* L = F.val + (long)q * bb;
    const V* yj = y + (long)F.idx[q] * b;
    for (int a = 0; a < b; ++a)
      for (int c = 0; c < b; ++c) acc[a] -= L[(long)a * b + c] * yj[c];
  }
  const V* D = F.val + (long)F.diag[i] * bb;
  for (int a = 0; a < b; ++a) {
    V s = acc[a];
    for (int c = 0; c < a; ++c) s -= D[(long)a * b + c] * acc[c];
    acc[a] = s;
    y[(long)i * b + a] = s;
  }
}

// Backward sweep (U x = y) for one level; x holds y on entry.  Per scalar row the upper entries
// are consumed in ascending column order (in-block first, then the blocks k > i), as in
// aquaflux/solve/_ilu0.pyx:143-147.
template <class V>
__global__ void k_ilu_upper(IluView<V> F, const int* rows, int count, V* x) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t], b = F.b;
  const long bb = (long)b * b;
  const V* D = F.val + (long)F.diag[i] * bb;
  V* xi = x + (long)i * b;
  for (int a = b - 1; a >= 0; --a) {
    V s = xi[a];
    for (int c = a + 1; c < b; ++c) s -= D[(long)a * b + c] * xi[c];
    for (int q = F.diag[i] + 1; q < F.ptr[i + 1]; ++q) {
      const V* U = F.val + (long)q * bb + (long)a * b;
      const V* xk = x + (long)F.idx[q] * b;
      for (int c = 0; c < b; ++c) s -= U[c] * xk[c];
    }
    xi[a] = s / D[(long)a * b + a];
  }
}

// Transposed sweeps use the transpose map: tptr/tidx/tblk list, for block column i, the rows j
// and block indices of the stored blocks (j, i).
// U^T z = r: forward over block columns; z_i = U_ii^-T (r_i - sum_{j<i} U_ji^T z_j).
template <class V>
__global__ void k_ilu_upper_t(IluView<V> F, const int* tptr, const int* tidx, const int* tblk,
                              const int* rows, int count, V* z) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t], b = F.b;
  const long bb = (long)b * b;
  V acc[8];
  for (int a = 0; a < b; ++a) acc[a] = z[(long)i * b + a];
  for (int q = tptr[i]; q < tptr[i + 1]; ++q) {
    const int j = tidx[q];
    if (j >= i) continue;
    const V* U = F.val + (long)tblk[q] * bb;  // block (j, i)
    const V* zj = z + (long)j * b;
    for (int a = 0; a < b; ++a)
      for (int c = 0; c < b; ++c) acc[a] -= U[(long)c * b + a] * zj[c];
  }
  const V* D = F.val + (long)F.diag[i] * bb;
  for (int a = 0; a < b; ++a) {
    V s = acc[a];
    for (int c = 0; c < a; ++c) s -= D[(long)c * b + a] * acc[c];
    s = s / D[(long)a * b + a];
    acc[a] = s;
    z[(long)i * b + a] = s;
  }
}

// L^T x = z: backward over block columns; x_i = L_ii^-T (z_i - sum_{k>i} L_ki^T x_k).  The
// contributions are taken in descending row order, the order of the reference's scatter form
// (aquaflux/solve/_ilu0.pyx:174-178).
template <class V>
__global__ void k_ilu_lower_t(IluView<V> F, const int* tptr, const int* tidx, const int* tblk,
                              const int* rows, int count, V* x) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= count) return;
  const int i = rows[t], b = F.b;
  const long bb = (long)b * b;
  const V* D = F.val + (long)F.diag[i] * bb;
  V* xi = x + (long)i * b;
  for (int a = b - 1; a >= 0; --a) {
    V s = xi[a];
    for (int q = tptr[i + 1] - 1; q >= tptr[i]; --q) {
      const int k = tidx[q];
      if (k <= i) continue;
      const V* L = F.val + (long)tblk[q] * bb;  // block (k, i)
      const V* xk = x + (long)k * b;
      for (int c = b - 1; c >= 0; --c) s -= L[(long)c * b + a] * xk[c];
    }
    for (int c = b - 1; c > a; --c) s -= D[(long)c * b + a] * xi[c];
    xi[a] = s;
  }
}

// ---- lane-group kernels: an 8-lane group per block row, lane a owns scalar row / column a of
// the block (b <= 8), so the b x b block work of a row runs on b lanes instead of one thread.
// Element-wise operation orders are those of the one-thread kernels above, except the forward
// solve's upper sweep, which subtracts the off-diagonal blocks before the in-block terms (the
// reference subtracts in ascending column order); b = 1 uses the one-thread kernels.
#define FV_LG 8
__device__ __forceinline__ unsigned lg_mask() { return 0xffu << ((threadIdx.x & 31) & ~(FV_LG - 1)); }

// Factor the block rows of one level, a group of FV_LG lanes per block row (lane a = row a of the
// block), with a compile-time block size: the row's lower block, the pivot row's diagonal block and
// each upper block it updates with are held in registers (vector loads), the diagonal block's pivot
// rows are shuffled from the lane that owns them.  Every entry sees the scalar elimination of
// k_ilu_factor_level in the same order, so the factors are bitwise the same.
template <class V, int B>
__global__ void k_ilu_factor_lgb(IluView<V> F, const int* rows, int count,
                                 unsigned long long* zero_flag) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / FV_LG;
  const int a = threadIdx.x & (FV_LG - 1);
  if (gid >= count) return;  // whole groups exit together
  const unsigned mask = lg_mask();
  const int i = rows[gid];
  const bool live = a < B;
  const int ar = live ? a : 0;  // row index of the lane's (possibly unused) loads
  constexpr long BB = (long)B * B;
  const int re = F.ptr[i + 1], di = F.diag[i];
  for (int q = F.ptr[i]; q < di; ++q) {
    const int j = F.idx[q];
    V* Lij = F.val + (long)q * BB;
    const V* Ujj = F.val + (long)F.diag[j] * BB;
    V L[B], U[B * B];
    load_seg<B>(Lij + (long)ar * B, L);
#pragma unroll
    for (int r = 0; r < B; ++r) {
      V row[B];
      load_seg<B>(Ujj + (long)r * B, row);
#pragma unroll
      for (int c = 0; c < B; ++c) U[r * B + c] = row[c];
    }
#pragma unroll
    for (int cb = 0; cb < B; ++cb) {
      const V piv = U[cb * B + cb];
      if (piv == V(0) && a == 0) note_zero_pivot(zero_flag, i * B, j * B + cb);
      const V l = L[cb] / piv;
      L[cb] = l;
#pragma unroll
      for (int c2 = cb + 1; c2 < B; ++c2) L[c2] -= l * U[cb * B + c2];
    }
    if (live) {
#pragma unroll
      for (int c = 0; c < B; ++c) Lij[(long)a * B + c] = L[c];
    }
    // A_ik -= L_ij A_jk for k > j present in both rows (merge of sorted column lists)
    int p = q + 1;
    for (int s2 = F.diag[j] + 1; s2 < F.ptr[j + 1]; ++s2) {
      const int k = F.idx[s2];
      while (p < re && F.idx[p] < k) ++p;
      if (p >= re) break;
      if (F.idx[p] != k) continue;
      V* Aik = F.val + (long)p * BB + (long)ar * B;
      const V* Ajk = F.val + (long)s2 * BB;
      V A[B], M[B * B];
      load_seg<B>(Aik, A);
#pragma unroll
      for (int r = 0; r < B; ++r) {
        V row[B];
        load_seg<B>(Ajk + (long)r * B, row);
#pragma unroll
        for (int c = 0; c < B; ++c) M[r * B + c] = row[c];
      }
#pragma unroll
      for (int c = 0; c < B; ++c) {
        V acc = A[c];
#pragma unroll
        for (int mm = 0; mm < B; ++mm) acc -= L[mm] * M[mm * B + c];
        A[c] = acc;
      }
      if (live) {
#pragma unroll
        for (int c = 0; c < B; ++c) Aik[c] = A[c];
      }
    }
  }
  __syncwarp(mask);
  V* D = F.val + (long)di * BB;
  V Drow[B];
  load_seg<B>(D + (long)ar * B, Drow);
#pragma unroll
  for (int cb = 0; cb < B; ++cb) {
    // row cb of the diagonal block is final: lane cb's registers; of the upper blocks: in memory
    V prow[B];
#pragma unroll
    for (int c = 0; c < B; ++c) prow[c] = __shfl_sync(mask, Drow[c], cb, FV_LG);
    if (live && a > cb) {
      const V piv = prow[cb];
      if (piv == V(0)) note_zero_pivot(zero_flag, i * B + a, i * B + cb);
      const V l = Drow[cb] / piv;
      Drow[cb] = l;
#pragma unroll
      for (int c = cb + 1; c < B; ++c) Drow[c] -= l * prow[c];
      for (int q = di + 1; q < re; ++q) {
        V* Ub = F.val + (long)q * BB;
        V ua[B], uc[B];
        load_seg<B>(Ub + (long)a * B, ua);
        load_seg<B>(Ub + (long)cb * B, uc);
#pragma unroll
        for (int c = 0; c < B; ++c) ua[c] -= l * uc[c];
#pragma unroll
        for (int c = 0; c < B; ++c) Ub[(long)a * B + c] = ua[c];
      }
    }
    __syncwarp(mask);
  }
  if (live) {
#pragma unroll
    for (int c = 0; c < B; ++c) D[(long)a * B + c] = Drow[c];
  }
}

// Forward sweep of one level, a group of FV_LG lanes per block row (lane a = row a of the block).
template <class V, int B>
__global__ void k_ilu_lower_lg(IluView<V> F, const int* rows, int count, V* y) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / FV_LG;
  const int a = threadIdx.x & (FV_LG - 1);
  if (gid >= count) return;
  const unsigned mask = lg_mask();
  const int i = rows[gid];
  const bool live = a < B;
  constexpr long BB = (long)B * B;
  V acc = live ? y[(long)i * B + a] : V(0);
  if (live)
    for (int q = F.ptr[i]; q < F.diag[i]; ++q) {
      V L[B], yj[B];
      load_seg<B>(F.val + (long)q * BB + (long)a * B, L);
      load_seg<B>(y + (long)F.idx[q] * B, yj);
#pragma unroll
      for (int c = 0; c < B; ++c) acc -= L[c] * yj[c];
    }
  V D[B];
  if (live) load_seg<B>(F.val + (long)F.diag[i] * BB + (long)a * B, D);
#pragma unroll
  for (int c = 0; c < B; ++c) {
    const V vc = __shfl_sync(mask, acc, c, FV_LG);
    if (live && a > c) acc -= D[c] * vc;
  }
  if (live) y[(long)i * B + a] = acc;
}

// The in-block upper solve of one block row (lane a holds entry a of the row's right-hand side,
// D the lane's row of the diagonal block).  Every lane forms the correctly rounded reciprocal r
// of its own pivot d up front (all lanes at once), so the dependent chain needs no division: a
// division there runs on one lane in eight at each step (fp32: 87 us of a 155 us diagonal-only
// sweep of 1M block rows under ncu; fp64: the 128^3 fine-level solve 6.5 ms with divisions,
// GB300).  The quotient x / d is q = x r corrected once, q + (x - q d) r, with fused
// multiply-adds: by Markstein's theorem (IBM J. Res. Develop. 34(1), 1990) the correctly rounded
// quotient, outside the underflow range (pinned bitwise against IEEE division in both precisions
// by the sparse-solver tests).  A lane whose reciprocal overflows (fp32 pivot below ~3e-39)
// divides.
template <class V, int B>
__device__ __forceinline__ V upper_block_solve(V acc, const V (&D)[B], int a, bool live,
                                               unsigned mask) {
  V piv = V(1);
#pragma unroll
  for (int c = 0; c < B; ++c)
    if (a == c) piv = D[c];
  const V rpiv = V(1) / piv;
  const bool rfin = isfinite(rpiv);
#pragma unroll
  for (int c = B - 1; c >= 0; --c) {
    if (a == c) {
      if (rfin) {
        const V q = acc * rpiv;
        acc = fma_rn(fma_rn(-q, piv, acc), rpiv, q);
      } else {
        acc = acc / piv;
      }
    }
    const V vc = __shfl_sync(mask, acc, c, FV_LG);
    if (live && a < c) acc -= D[c] * vc;
  }
  return acc;
}

// Backward sweep of one level (U x = y).
template <class V, int B>
__global__ void k_ilu_upper_lg(IluView<V> F, const int* rows, int count, V* x) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / FV_LG;
  const int a = threadIdx.x & (FV_LG - 1);
  if (gid >= count) return;
  const unsigned mask = lg_mask();
  const int i = rows[gid];
  const bool live = a < B;
  constexpr long BB = (long)B * B;
  V acc = live ? x[(long)i * B + a] : V(0);
  if (live)
    for (int q = F.diag[i] + 1; q < F.ptr[i + 1]; ++q) {
      V U[B], xk[B];
      load_seg<B>(F.val + (long)q * BB + (long)a * B, U);
      load_seg<B>(x + (long)F.idx[q] * B, xk);
#pragma unroll
      for (int c = 0; c < B; ++c) acc -= U[c] * xk[c];
    }
  V D[B];
  if (live) load_seg<B>(F.val + (long)F.diag[i] * BB + (long)a * B, D);
  acc = upper_block_solve<V, B>(acc, D, a, live, mask);
  if (live) x[(long)i * B + a] = acc;
}

// The last forward level followed by the first backward level on the same rows, one kernel: when
// those rows own no upper blocks (the second colour of a two-colour order), a row's backward step
// is the in-block upper solve of its own forward result, with the diagonal block already in
// registers.  The same operations in the same order as the two separate sweeps.
template <class V, int B>
__global__ void k_ilu_lower_upper_lg(IluView<V> F, const int* rows, int count, V* y) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / FV_LG;
  const int a = threadIdx.x & (FV_LG - 1);
  if (gid >= count) return;
  const unsigned mask = lg_mask();
  const int i = rows[gid];
  const bool live = a < B;
  constexpr long BB = (long)B * B;
  V acc = live ? y[(long)i * B + a] : V(0);
  if (live)
    for (int q = F.ptr[i]; q < F.diag[i]; ++q) {
      V L[B], yj[B];
      load_seg<B>(F.val + (long)q * BB + (long)a * B, L);
      load_seg<B>(y + (long)F.idx[q] * B, yj);
#pragma unroll
      for (int c = 0; c < B; ++c) acc -= L[c] * yj[c];
    }
  V D[B];
  if (live) load_seg<B>(F.val + (long)F.diag[i] * BB + (long)a * B, D);
#pragma unroll
  for (int c = 0; c < B; ++c) {
    const V vc = __shfl_sync(mask, acc, c, FV_LG);
    if (live && a > c) acc -= D[c] * vc;
  }
  acc = upper_block_solve<V, B>(acc, D, a, live, mask);
  if (live) y[(long)i * B + a] = acc;
}

// The in-block lower solve of U^T's diagonal block D^T (lane a holds entry a of the right-hand
// side, Dc the lane's column of D: Dc[c] = D(c, a)): step c divides entry c by its pivot D(c, c),
// then every later entry a > c takes -D(c, a) times it.  The division is the reciprocal quotient
// of upper_block_solve (every lane's reciprocal formed up front, one fused correction: the
// correctly rounded quotient, the same value as the division).
template <class V, int B>
__device__ __forceinline__ V lower_t_block_solve(V acc, const V (&Dc)[B], int a, bool live,
                                                 unsigned mask) {
  V piv = V(1);
#pragma unroll
  for (int c = 0; c < B; ++c)
    if (a == c) piv = Dc[c];
  const V rpiv = V(1) / piv;
  const bool rfin = isfinite(rpiv);
#pragma unroll
  for (int c = 0; c < B; ++c) {
    if (a == c) {
      if (rfin) {
        const V q = acc * rpiv;
        acc = fma_rn(fma_rn(-q, piv, acc), rpiv, q);
      } else {
        acc = acc / piv;
      }
    }
    const V vc = __shfl_sync(mask, acc, c, FV_LG);
    if (live && a > c) acc -= Dc[c] * vc;
  }
  return acc;
}

// Forward sweep of one level of the transposed solve, U^T z = r: block row i of U^T takes the
// blocks (j, i) of U, j < i (positions tptr[i] .. tdiag[i] of the transpose, ascending j), row a
// of each transposed block (column a of the block of U) for lane a, then the in-block lower solve
// with D^T -- the operations and their order of the reference's transposed solve.
template <class V, int B>
__global__ void k_ilu_upper_t_lg(IluView<V> F, const int* tptr, const int* tidx, const int* tdiag,
                                 const V* tval, const int* rows, int count, V* z) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / FV_LG;
  const int a = threadIdx.x & (FV_LG - 1);
  if (gid >= count) return;
  const unsigned mask = lg_mask();
  const int i = rows[gid];
  const bool live = a < B;
  constexpr long BB = (long)B * B;
  V acc = live ? z[(long)i * B + a] : V(0);
  if (live)
    for (int q = tptr[i]; q < tdiag[i]; ++q) {
      V Ut[B], zj[B];
      load_seg<B>(tval + (long)q * BB + (long)a * B, Ut);
      load_seg<B>(z + (long)tidx[q] * B, zj);
#pragma unroll
      for (int c = 0; c < B; ++c) acc -= Ut[c] * zj[c];
    }
  V Dc[B];  // Dc[c] = D(c, a): row a of D^T
  if (live) load_seg<B>(tval + (long)tdiag[i] * BB + (long)a * B, Dc);
  else
#pragma unroll
    for (int c = 0; c < B; ++c) Dc[c] = V(0);
  acc = lower_t_block_solve<V, B>(acc, Dc, a, live, mask);
  if (live) z[(long)i * B + a] = acc;
}

// Backward sweep of one level of the transposed solve, L^T x = z (unit diagonal): the blocks
// (k, i) of L, k > i (positions tptr[i + 1] - 1 down to tdiag[i] + 1), then the in-block unit
// upper solve.
template <class V, int B>
__global__ void k_ilu_lower_t_lg(IluView<V> F, const int* tptr, const int* tidx, const int* tdiag,
                                 const V* tval, const int* rows, int count, V* x) {
  const int gid = (blockIdx.x * blockDim.x + threadIdx.x) / FV_LG;
  const int a = threadIdx.x & (FV_LG - 1);
  if (gid >= count) return;
  const unsigned mask = lg_mask();
  const int i = rows[gid];
  const bool live = a < B;
  constexpr long BB = (long)B * B;
  V acc = live ? x[(long)i * B + a] : V(0);
  if (live)
    for (int q = tptr[i + 1] - 1; q > tdiag[i]; --q) {
      V Lt[B], xk[B];
      load_seg<B>(tval + (long)q * BB + (long)a * B, Lt);
      load_seg<B>(x + (long)tidx[q] * B, xk);
#pragma unroll
      for (int c = B - 1; c >= 0; --c) acc -= Lt[c] * xk[c];
    }
  V Dc[B];
  if (live) load_seg<B>(tval + (long)tdiag[i] * BB + (long)a * B, Dc);
  else
#pragma unroll
    for (int c = 0; c < B; ++c) Dc[c] = V(0);
#pragma unroll
  for (int c = B - 1; c >= 0; --c) {
    const V vc = __shfl_sync(mask, acc, c, FV_LG);
    if (live && a < c) acc -= Dc[c] * vc;
  }
  if (live) x[(long)i * B + a] = acc;
}

template <class V>
__global__ void k_copy(long n, const V* a, V* b) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}
__global__ void k_to_f32(long n, const double* a, float* b) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

// ------------------------------------------------------------------------------ reductions
constexpr int kRedBlocks = 304;  // 2 x 152 SMs, fixed so the summation order never changes
__global__ void k_dot_partial(long n, const double* x, const double* y, double* part) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
    s += x[i] * y[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}
__global__ void k_dot_final(int nparts, const double* part, double* out) {
  __shared__ double sh[kThreads];
  double s = 0.0;
  for (int i = threadIdx.x; i < nparts; i += blockDim.x) s += part[i];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

double* g_dot_parts = nullptr;

}  // namespace

// ------------------------------------------------------------------------------ FvIlu0
struct FvIlu0 {
  int n = 0, b = 0, nnzb = 0, precision = 64;
  int *ptr = nullptr, *idx = nullptr, *diag = nullptr;
  int *tptr = nullptr, *tidx = nullptr, *tblk = nullptr;
  int* tdiag = nullptr;   // position of the diagonal block in each row of the transpose
  void* val = nullptr;
  void* tval = nullptr;   // (b > 1) the factor's blocks transposed, in the transpose's order
  unsigned long long* zero_flag = nullptr;
  // level sets: rows grouped by level (device), level boundaries (host)
  int* rows_fwd = nullptr;   // L / factor order
  int* rows_bwd = nullptr;   // U order (from the last row)
  int* rows_tfwd = nullptr;  // U^T order
  int* rows_tbwd = nullptr;  // L^T order
  std::vector<int> lv_fwd, lv_bwd, lv_tfwd, lv_tbwd;
  void* work = nullptr;                      // (n * b) vector the captured sweeps run on
  bool fuse_fb = false;  // the last forward level's rows are the first backward level's (fused)
  cudaGraphExec_t apply_exec[2] = {nullptr, nullptr};  // forward / transposed solve
  cudaGraphExec_t factor_exec = nullptr;
  // host copy of the pattern (shared by clones): the transposed-solve structures are built on
  // first use
  std::shared_ptr<const std::vector<int>> h_ptr, h_idx, h_diag;
};

namespace {

// Level sets of a dependency DAG given as "row i depends on rows deps(i)".
template <class DepFn>
void levels(int n, bool ascending, DepFn deps, std::vector<int>* rows, std::vector<int>* bounds) {
  std::vector<int> lev(n, 0);
  int maxl = 0;
  if (ascending) {
    for (int i = 0; i < n; ++i) {
      int l = 0;
      deps(i, [&](int j) { l = std::max(l, lev[j] + 1); });
      lev[i] = l;
      maxl = std::max(maxl, l);
    }
  } else {
    for (int i = n - 1; i >= 0; --i) {
      int l = 0;
      deps(i, [&](int j) { l = std::max(l, lev[j] + 1); });
      lev[i] = l;
      maxl = std::max(maxl, l);
    }
  }
  bounds->assign(maxl + 2, 0);
  for (int i = 0; i < n; ++i) (*bounds)[lev[i] + 1]++;
  for (int l = 0; l <= maxl; ++l) (*bounds)[l + 1] += (*bounds)[l];
  rows->assign(n, 0);
  std::vector<int> fill(bounds->begin(), bounds->end() - 1);
  for (int i = 0; i < n; ++i) (*rows)[fill[lev[i]]++] = i;
}

template <class V>
IluView<V> view(FvIlu0* f) {
  return IluView<V>{f->n, f->b, f->ptr, f->idx, f->diag, (V*)f->val};
}

// Launch the level sequence of the factorization / a solve on `s` (captured into a graph once).
template <class V>
void launch_factor_levels(FvIlu0* f, cudaStream_t s) {
  IluView<V> F = view<V>(f);
  for (size_t l = 0; l + 1 < f->lv_fwd.size(); ++l) {
    const int cnt = f->lv_fwd[l + 1] - f->lv_fwd[l];
    if (cnt == 0) continue;
    if (f->b == 1)
      k_ilu_factor_level<V><<<fv_blocks(cnt, 128), 128, 0, s>>>(F, f->rows_fwd + f->lv_fwd[l], cnt,
                                                                f->zero_flag);
    else
      with_block_size(f->b, [&](auto B) {
        k_ilu_factor_lgb<V, B()><<<fv_blocks((long)cnt * FV_LG, 128), 128, 0, s>>>(
            F, f->rows_fwd + f->lv_fwd[l], cnt, f->zero_flag);
      });
  }
}

template <class V>
void launch_apply_levels(FvIlu0* f, int transpose, V* x, cudaStream_t s) {
  IluView<V> F = view<V>(f);
  const bool lg = f->b > 1;
  auto grid = [&](int cnt) { return lg ? fv_blocks((long)cnt * FV_LG, 128) : fv_blocks(cnt, 128); };
  if (!transpose) {
    const size_t last = f->lv_fwd.size() - 2;
    for (size_t l = 0; l + 1 < f->lv_fwd.size(); ++l) {
      const int cnt = f->lv_fwd[l + 1] - f->lv_fwd[l];
      if (!cnt) continue;
      if (lg && f->fuse_fb && l == last)
        with_block_size(f->b, [&](auto B) {
          k_ilu_lower_upper_lg<V, B()><<<grid(cnt), 128, 0, s>>>(F, f->rows_fwd + f->lv_fwd[l],
                                                                 cnt, x);
        });
      else if (lg)
        with_block_size(f->b, [&](auto B) {
          k_ilu_lower_lg<V, B()><<<grid(cnt), 128, 0, s>>>(F, f->rows_fwd + f->lv_fwd[l], cnt, x);
        });
      else k_ilu_lower<V><<<grid(cnt), 128, 0, s>>>(F, f->rows_fwd + f->lv_fwd[l], cnt, x);
    }
    for (size_t l = f->fuse_fb ? 1 : 0; l + 1 < f->lv_bwd.size(); ++l) {
      const int cnt = f->lv_bwd[l + 1] - f->lv_bwd[l];
      if (!cnt) continue;
      if (lg)
        with_block_size(f->b, [&](auto B) {
          k_ilu_upper_lg<V, B()><<<grid(cnt), 128, 0, s>>>(F, f->rows_bwd + f->lv_bwd[l], cnt, x);
        });
      else k_ilu_upper<V><<<grid(cnt), 128, 0, s>>>(F, f->rows_bwd + f->lv_bwd[l], cnt, x);
    }
  } else {
    for (size_t l = 0; l + 1 < f->lv_tfwd.size(); ++l) {
      const int cnt = f->lv_tfwd[l + 1] - f->lv_tfwd[l];
      if (!cnt) continue;
      const int* rows = f->rows_tfwd + f->lv_tfwd[l];
      if (lg)
        with_block_size(f->b, [&](auto B) {
          k_ilu_upper_t_lg<V, B()><<<grid(cnt), 128, 0, s>>>(F, f->tptr, f->tidx, f->tdiag,
                                                             (const V*)f->tval, rows, cnt, x);
        });
      else k_ilu_upper_t<V><<<grid(cnt), 128, 0, s>>>(F, f->tptr, f->tidx, f->tblk, rows, cnt, x);
    }
    for (size_t l = 0; l + 1 < f->lv_tbwd.size(); ++l) {
      const int cnt = f->lv_tbwd[l + 1] - f->lv_tbwd[l];
      if (!cnt) continue;
      const int* rows = f->rows_tbwd + f->lv_tbwd[l];
      if (lg)
        with_block_size(f->b, [&](auto B) {
          k_ilu_lower_t_lg<V, B()><<<grid(cnt), 128, 0, s>>>(F, f->tptr, f->tidx, f->tdiag,
                                                             (const V*)f->tval, rows, cnt, x);
        });
      else k_ilu_lower_t<V><<<grid(cnt), 128, 0, s>>>(F, f->tptr, f->tidx, f->tblk, rows, cnt, x);
    }
  }
}

// Capture `body` (a sequence of launches on a stream) into an executable graph, on a private
// stream in thread-local capture mode so that a caller's own capture is unaffected.
template <class Body>
int capture(Body body, cudaGraphExec_t* out) {
  cudaStream_t cs;
  FV_CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  cudaGraph_t g = nullptr;
  cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
  if (e == cudaSuccess) {
    body(cs);
    e = cudaStreamEndCapture(cs, &g);
  }
  if (e == cudaSuccess) e = cudaGraphInstantiate(out, g, 0);
  if (g) cudaGraphDestroy(g);
  cudaStreamDestroy(cs);
  if (e != cudaSuccess) {
    fv_set_error("ILU(0) graph capture failed: %s", cudaGetErrorString(e));
    return FV_ERR_CUDA;
  }
  return FV_OK;
}

template <class V>
int ilu_factor(FvIlu0* f, cudaStream_t s) {
  unsigned long long init = ~0ull;
  FV_CUDA_TRY(cudaMemcpyAsync(f->zero_flag, &init, sizeof(init), cudaMemcpyHostToDevice, s));
  if (!f->factor_exec) {
    int rc = capture([&](cudaStream_t cs) { launch_factor_levels<V>(f, cs); }, &f->factor_exec);
    if (rc != FV_OK) return rc;
  }
  FV_CUDA_TRY(cudaGraphLaunch(f->factor_exec, s));
  if (f->tval) {  // a transposed solve was asked for: keep its transposed blocks current
    const long nv = (long)f->nnzb * f->b * f->b;
    k_transpose_blocks<V><<<fv_blocks(nv, kThreads), kThreads, 0, s>>>(f->nnzb, f->b, f->tblk,
                                                                      (const V*)f->val,
                                                                      (V*)f->tval);
  }
  FV_CUDA_TRY(cudaGetLastError());
  unsigned long long flag;
  FV_CUDA_TRY(cudaMemcpyAsync(&flag, f->zero_flag, sizeof(flag), cudaMemcpyDeviceToHost, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  if (flag != ~0ull) {
    long col = (long)(flag & 0xffffffffull);
    fv_set_error_index(col);
    fv_set_error(
        "ILU(0) met an exactly zero pivot at row %ld; the operator needs a different ordering or "
        "an explicit shift, neither of which this routine applies silently.",
        col);
    return FV_ERR_ZERO_PIVOT;
  }
  return FV_OK;
}

int upload(const std::vector<int>& h, int** d, cudaStream_t s);

// The transposed-solve structures (the pattern's transpose and the level sets of U^T and L^T),
// built the first time a transposed solve is asked for.
int ensure_transpose(FvIlu0* f, cudaStream_t s) {
  if (f->tptr) return FV_OK;
  const int n = f->n;
  Transpose T;
  build_transpose(n, n, f->h_ptr->data(), f->h_idx->data(), &T);
  std::vector<int> rows;
  levels(n, true, [&](int i, auto&& use) {  // U^T: column i depends on rows j < i with (j, i)
    for (int q = T.ptr[i]; q < T.ptr[i + 1]; ++q)
      if (T.idx[q] < i) use(T.idx[q]);
  }, &rows, &f->lv_tfwd);
  if (upload(rows, &f->rows_tfwd, s)) return FV_ERR_CUDA;
  levels(n, false, [&](int i, auto&& use) {  // L^T: column i depends on rows k > i with (k, i)
    for (int q = T.ptr[i]; q < T.ptr[i + 1]; ++q)
      if (T.idx[q] > i) use(T.idx[q]);
  }, &rows, &f->lv_tbwd);
  if (upload(rows, &f->rows_tbwd, s)) return FV_ERR_CUDA;
  if (upload(T.ptr, &f->tptr, s) || upload(T.idx, &f->tidx, s) || upload(T.blk, &f->tblk, s))
    return FV_ERR_CUDA;
  if (f->b > 1) {  // the lane-group sweeps read the factor's blocks transposed
    std::vector<int> td(n, -1);
    for (int i = 0; i < n; ++i)
      for (int q = T.ptr[i]; q < T.ptr[i + 1]; ++q)
        if (T.idx[q] == i) td[i] = q;
    if (upload(td, &f->tdiag, s)) return FV_ERR_CUDA;
    const long nv = (long)f->nnzb * f->b * f->b;
    const size_t vs = f->precision == 64 ? sizeof(double) : sizeof(float);
    FV_CUDA_TRY(cudaMalloc(&f->tval, vs * (size_t)nv));
    if (f->precision == 64)
      k_transpose_blocks<double><<<fv_blocks(nv, kThreads), kThreads, 0, s>>>(
          f->nnzb, f->b, f->tblk, (const double*)f->val, (double*)f->tval);
    else
      k_transpose_blocks<float><<<fv_blocks(nv, kThreads), kThreads, 0, s>>>(
          f->nnzb, f->b, f->tblk, (const float*)f->val, (float*)f->tval);
    FV_CUDA_TRY(cudaGetLastError());
  }
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  return FV_OK;
}

template <class V>
int ilu_apply(FvIlu0* f, const V* r, V* x, int transpose, cudaStream_t s) {
  const long n = (long)f->n * f->b;
  V* w = (V*)f->work;
  const int t = transpose ? 1 : 0;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  FV_CUDA_TRY(cudaStreamIsCapturing(s, &cap));
  if (cap != cudaStreamCaptureStatusNone) {
    // inside a caller's stream capture (a whole V-cycle as one graph): the level kernels go
    // straight into the caller's graph and run in place on x; nothing is allocated or built here
    if (t && !f->tptr) {
      fv_set_error("fv_ilu0_apply: the transposed-solve structures are built by a transposed "
                   "solve outside stream capture first");
      return FV_ERR_ARG;
    }
    if ((uintptr_t)x % 16 != 0) {  // the level kernels read x's block segments as vectors
      fv_set_error("fv_ilu0_apply: under stream capture x must be 16-byte aligned");
      return FV_ERR_ARG;
    }
    if ((const void*)x != (const void*)r)
      FV_CUDA_TRY(cudaMemcpyAsync(x, r, sizeof(V) * n, cudaMemcpyDeviceToDevice, s));
    launch_apply_levels<V>(f, t, x, s);
    FV_CUDA_TRY(cudaGetLastError());
    return FV_OK;
  }
  if (t) {
    int rc = ensure_transpose(f, s);
    if (rc != FV_OK) return rc;
  }
  if (!f->apply_exec[t]) {
    int rc = capture([&](cudaStream_t cs) { launch_apply_levels<V>(f, t, w, cs); },
                     &f->apply_exec[t]);
    if (rc != FV_OK) return rc;
  }
  FV_CUDA_TRY(cudaMemcpyAsync(w, r, sizeof(V) * n, cudaMemcpyDeviceToDevice, s));
  FV_CUDA_TRY(cudaGraphLaunch(f->apply_exec[t], s));
  FV_CUDA_TRY(cudaMemcpyAsync(x, w, sizeof(V) * n, cudaMemcpyDeviceToDevice, s));
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

int upload(const std::vector<int>& h, int** d, cudaStream_t s) {
  FV_CUDA_TRY(cudaMalloc(d, sizeof(int) * std::max<size_t>(1, h.size())));
  if (!h.empty())
    FV_CUDA_TRY(cudaMemcpyAsync(*d, h.data(), sizeof(int) * h.size(), cudaMemcpyHostToDevice, s));
  return FV_OK;
}

}  // namespace

extern "C" int fv_ilu0_create(int n, int b, const int* indptr, const int* indices, int precision,
                              void* stream, FvIlu0** out) {
  if (!out || n <= 0 || b <= 0 || b > 8 || !indptr || !indices ||
      (precision != 32 && precision != 64)) {
    fv_set_error("fv_ilu0_create: bad arguments (1 <= b <= 8, precision 32 or 64)");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const int nnzb = indptr[n];
  std::vector<int> diag(n, -1);
  for (int i = 0; i < n; ++i) {
    for (int q = indptr[i]; q < indptr[i + 1]; ++q) {
      if (indices[q] < 0 || indices[q] >= n || (q > indptr[i] && indices[q] <= indices[q - 1])) {
        fv_set_error("fv_ilu0_create: row %d has unsorted or out-of-range column indices", i);
        return FV_ERR_ARG;
      }
      if (indices[q] == i) diag[i] = q;
    }
  }
  // reference message: aquaflux/solve/_ilu0.pyx:56-63 (the first rows missing a diagonal)
  std::vector<int> missing;
  for (int i = 0; i < n; ++i)
    if (diag[i] < 0) missing.push_back(i);
  if (!missing.empty()) {
    char buf[256];
    int len = snprintf(buf, sizeof(buf), "rows [");
    for (size_t k = 0; k < missing.size() && k < 5; ++k)
      len += snprintf(buf + len, sizeof(buf) - len, "%s%d", k ? ", " : "", missing[k] * b);
    snprintf(buf + len, sizeof(buf) - len, "]%s", missing.size() > 5 ? " \xe2\x80\xa6" : "");
    fv_set_error_index((long)missing[0] * b);
    fv_set_error("%s store no diagonal entry; ILU(0) eliminates in place and cannot introduce one.",
                 buf);
    return FV_ERR_NO_DIAG;
  }
  FvIlu0* f = new FvIlu0();
  f->n = n;
  f->b = b;
  f->nnzb = nnzb;
  f->precision = precision;
  std::vector<int> rows;
  levels(n, true, [&](int i, auto&& use) {
    for (int q = indptr[i]; q < diag[i]; ++q) use(indices[q]);
  }, &rows, &f->lv_fwd);
  if (upload(rows, &f->rows_fwd, s)) return FV_ERR_CUDA;
  const size_t nf = f->lv_fwd.size();
  std::vector<int> fwd_last(rows.begin() + f->lv_fwd[nf - 2], rows.begin() + f->lv_fwd[nf - 1]);
  levels(n, false, [&](int i, auto&& use) {
    for (int q = diag[i] + 1; q < indptr[i + 1]; ++q) use(indices[q]);
  }, &rows, &f->lv_bwd);
  if (upload(rows, &f->rows_bwd, s)) return FV_ERR_CUDA;
  // fused last forward / first backward level when they hold the same rows (the first backward
  // level's rows own no upper blocks by construction)
  std::vector<int> bwd_first(rows.begin() + f->lv_bwd[0], rows.begin() + f->lv_bwd[1]);
  std::sort(fwd_last.begin(), fwd_last.end());
  std::sort(bwd_first.begin(), bwd_first.end());
  f->fuse_fb = b > 1 && nf > 2 && f->lv_bwd.size() > 2 && fwd_last == bwd_first;
  f->h_ptr = std::make_shared<const std::vector<int>>(indptr, indptr + n + 1);
  f->h_idx = std::make_shared<const std::vector<int>>(indices, indices + nnzb);
  f->h_diag = std::make_shared<const std::vector<int>>(diag);
  if (upload(*f->h_ptr, &f->ptr, s) || upload(*f->h_idx, &f->idx, s) || upload(diag, &f->diag, s))
    return FV_ERR_CUDA;
  size_t vs = precision == 64 ? sizeof(double) : sizeof(float);
  FV_CUDA_TRY(cudaMalloc(&f->val, vs * (size_t)nnzb * b * b));
  FV_CUDA_TRY(cudaMalloc(&f->zero_flag, sizeof(unsigned long long)));
  FV_CUDA_TRY(cudaMalloc(&f->work, vs * (size_t)n * b));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  *out = f;
  return FV_OK;
}

extern "C" int fv_ilu0_destroy(FvIlu0* f) {
  if (!f) return FV_OK;
  cudaFree(f->ptr);
  cudaFree(f->idx);
  cudaFree(f->diag);
  cudaFree(f->tptr);
  cudaFree(f->tidx);
  cudaFree(f->tblk);
  cudaFree(f->tdiag);
  cudaFree(f->val);
  cudaFree(f->tval);
  cudaFree(f->zero_flag);
  cudaFree(f->rows_fwd);
  cudaFree(f->rows_bwd);
  cudaFree(f->rows_tfwd);
  cudaFree(f->rows_tbwd);
  cudaFree(f->work);
  for (cudaGraphExec_t e : f->apply_exec)
    if (e) cudaGraphExecDestroy(e);
  if (f->factor_exec) cudaGraphExecDestroy(f->factor_exec);
  delete f;
  return FV_OK;
}

namespace {
// Device copy of n ints (nothing when the source is absent).
int copy_ints(const int* src, size_t n, int** dst, cudaStream_t s) {
  if (!src) return FV_OK;
  FV_CUDA_TRY(cudaMalloc(dst, sizeof(int) * std::max<size_t>(1, n)));
  FV_CUDA_TRY(cudaMemcpyAsync(*dst, src, sizeof(int) * n, cudaMemcpyDeviceToDevice, s));
  return FV_OK;
}
}  // namespace

extern "C" int fv_ilu0_clone(const FvIlu0* src, int precision, void* stream, FvIlu0** out) {
  if (!src || !out || (precision != 0 && precision != 32 && precision != 64)) {
    fv_set_error("fv_ilu0_clone: bad arguments (precision 0, 32 or 64)");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  FvIlu0* f = new FvIlu0();
  f->n = src->n;
  f->b = src->b;
  f->nnzb = src->nnzb;
  f->precision = precision;
  f->lv_fwd = src->lv_fwd;
  f->lv_bwd = src->lv_bwd;
  f->lv_tfwd = src->lv_tfwd;
  f->lv_tbwd = src->lv_tbwd;
  f->fuse_fb = src->fuse_fb;
  f->h_ptr = src->h_ptr;
  f->h_idx = src->h_idx;
  f->h_diag = src->h_diag;
  const size_t n = src->n, nnzb = src->nnzb;
  int rc = FV_OK;
  rc |= copy_ints(src->ptr, n + 1, &f->ptr, s);
  rc |= copy_ints(src->idx, nnzb, &f->idx, s);
  rc |= copy_ints(src->diag, n, &f->diag, s);
  rc |= copy_ints(src->rows_fwd, n, &f->rows_fwd, s);
  rc |= copy_ints(src->rows_bwd, n, &f->rows_bwd, s);
  if (src->tptr) {
    rc |= copy_ints(src->tptr, n + 1, &f->tptr, s);
    rc |= copy_ints(src->tidx, nnzb, &f->tidx, s);
    rc |= copy_ints(src->tblk, nnzb, &f->tblk, s);
    rc |= copy_ints(src->rows_tfwd, n, &f->rows_tfwd, s);
    rc |= copy_ints(src->rows_tbwd, n, &f->rows_tbwd, s);
    rc |= copy_ints(src->tdiag, n, &f->tdiag, s);
  }
  if (rc == FV_OK && precision != 0) {
    const size_t vs = precision == 64 ? sizeof(double) : sizeof(float);
    if (cudaMalloc(&f->val, vs * nnzb * f->b * f->b) != cudaSuccess ||
        cudaMalloc(&f->zero_flag, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&f->work, vs * n * f->b) != cudaSuccess)
      rc = FV_ERR_CUDA;
    // the transposed blocks, filled by the clone's factorisations
    if (rc == FV_OK && f->tdiag && cudaMalloc(&f->tval, vs * nnzb * f->b * f->b) != cudaSuccess)
      rc = FV_ERR_CUDA;
  }
  if (rc == FV_OK && cudaStreamSynchronize(s) != cudaSuccess) rc = FV_ERR_CUDA;
  if (rc != FV_OK) {
    fv_set_error("fv_ilu0_clone: device allocation or copy failed");
    fv_ilu0_destroy(f);
    return FV_ERR_CUDA;
  }
  *out = f;
  return FV_OK;
}

extern "C" int fv_ilu0_factor(FvIlu0* f, const void* values, int values_f64, void* stream) {
  if (!f || !values || !f->val) {
    fv_set_error("fv_ilu0_factor: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long n = (long)f->nnzb * f->b * f->b;
  if (f->precision == 64) {
    FV_CUDA_TRY(cudaMemcpyAsync(f->val, values, sizeof(double) * n, cudaMemcpyDeviceToDevice, s));
    return ilu_factor<double>(f, s);
  }
  if (values_f64)
    k_to_f32<<<fv_blocks(n, kThreads), kThreads, 0, s>>>(n, (const double*)values, (float*)f->val);
  else
    FV_CUDA_TRY(cudaMemcpyAsync(f->val, values, sizeof(float) * n, cudaMemcpyDeviceToDevice, s));
  return ilu_factor<float>(f, s);
}

extern "C" int fv_ilu0_apply(FvIlu0* f, const void* r, void* x, int transpose, void* stream) {
  if (!f || !r || !x || !f->val) {
    fv_set_error("fv_ilu0_apply: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (f->precision == 64) return ilu_apply<double>(f, (const double*)r, (double*)x, transpose, s);
  return ilu_apply<float>(f, (const float*)r, (float*)x, transpose, s);
}

extern "C" int fv_ilu0_factor_values(const FvIlu0* f, void* out, void* stream) {
  if (!f || !out || !f->val) {
    fv_set_error("fv_ilu0_factor_values: bad arguments");
    return FV_ERR_ARG;
  }
  size_t vs = f->precision == 64 ? sizeof(double) : sizeof(float);
  FV_CUDA_TRY(cudaMemcpyAsync(out, f->val, vs * (size_t)f->nnzb * f->b * f->b,
                              cudaMemcpyDeviceToDevice, (cudaStream_t)stream));
  return FV_OK;
}

// ------------------------------------------------------------------------------ shifted operator
namespace {
// Diagonal of every dof (cell i, field a) after the shift, and its equilibration factor.
__global__ void k_shift_diag(int n, int b, const int* __restrict__ ptr, const int* __restrict__ idx,
                             const double* __restrict__ val, const double* __restrict__ shift,
                             double* diag_cm, double* scale_cm, double* scale_fm, int* missing) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * b) return;
  const int i = (int)(t / b), a = (int)(t % b);
  int dq = -1;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q)
    if (idx[q] == i) {
      dq = q;
      break;
    }
  if (dq < 0) {
    atomicMin(missing, i);
    return;
  }
  double d = val[((long)dq * b + a) * b + a];
  if (shift) d = d + shift[(long)a * n + i];
  diag_cm[t] = d;
  if (scale_cm) {
    double m = fabs(d);
    if (m == 0.0) m = 1.0;
    const double sc = 1.0 / sqrt(m);
    scale_cm[t] = sc;
    if (scale_fm) scale_fm[(long)a * n + i] = sc;
  }
}

// out[q][a][c] = ((v + shift on the diagonal) * s_row) * s_col, one thread per scalar row (i, a).
template <class Out>
__global__ void k_shift_scale(int n, int b, const int* __restrict__ ptr, const int* __restrict__ idx,
                              const double* __restrict__ val, const double* __restrict__ diag_cm,
                              const double* __restrict__ scale_cm, Out* __restrict__ out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * b) return;
  const int i = (int)(t / b), a = (int)(t % b);
  const double sr = scale_cm ? scale_cm[t] : 1.0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    const int j = idx[q];
    const long base = ((long)q * b + a) * b;
    for (int c = 0; c < b; ++c) {
      double v = (j == i && c == a) ? diag_cm[t] : val[base + c];
      if (scale_cm) {
        v = v * sr;
        v = v * scale_cm[(long)j * b + c];
      }
      out[base + c] = (Out)v;
    }
  }
}
}  // namespace

extern "C" int fv_bsr_shift_equilibrate(int n, int b, const int* indptr, const int* indices,
                                        const double* values, const double* shift, int equilibrate,
                                        double* scale_fm, double* work, void* out, int out_f64,
                                        void* stream) {
  if (n <= 0 || b <= 0 || !indptr || !indices || !values || !work || !out) {
    fv_set_error("fv_bsr_shift_equilibrate: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long m = (long)n * b;
  double* diag_cm = work;
  double* scale_cm = equilibrate ? work + m : nullptr;
  int* missing = reinterpret_cast<int*>(work + 2 * m);
  const int init = 0x7fffffff;
  FV_CUDA_TRY(cudaMemcpyAsync(missing, &init, sizeof(int), cudaMemcpyHostToDevice, s));
  k_shift_diag<<<fv_blocks(m, kThreads), kThreads, 0, s>>>(n, b, indptr, indices, values, shift,
                                                           diag_cm, scale_cm, scale_fm, missing);
  if (out_f64)
    k_shift_scale<double><<<fv_blocks(m, kThreads), kThreads, 0, s>>>(
        n, b, indptr, indices, values, diag_cm, scale_cm, (double*)out);
  else
    k_shift_scale<float><<<fv_blocks(m, kThreads), kThreads, 0, s>>>(
        n, b, indptr, indices, values, diag_cm, scale_cm, (float*)out);
  FV_CUDA_TRY(cudaGetLastError());
  int miss = 0;
  FV_CUDA_TRY(cudaMemcpyAsync(&miss, missing, sizeof(int), cudaMemcpyDeviceToHost, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  if (miss != init) {
    fv_set_error_index(miss);
    fv_set_error("fv_bsr_shift_equilibrate: block row %d stores no diagonal block; the shift has "
                 "nowhere to go", miss);
    return FV_ERR_NO_DIAG;
  }
  return FV_OK;
}

// ------------------------------------------------------------------------------ SpMV entry points
namespace {
template <class V>
int spmv(int nbr, int b, const int* indptr, const int* indices, const V* values, const V* x, V* y,
         int transpose, cudaStream_t s) {
  if (nbr <= 0 || b <= 0 || !indptr || !indices || !values || !x || !y) {
    fv_set_error("fv_bsr_spmv: bad arguments");
    return FV_ERR_ARG;
  }
  const long rows = (long)nbr * b;
  if (!transpose) {
    const bool aligned = ((uintptr_t)values % 16 == 0) && ((uintptr_t)x % 16 == 0);
    if (aligned && b >= 2 && b <= 8)
      with_block_size(b, [&](auto B) {
        k_bsr_spmv_b<V, B()><<<fv_blocks(rows, kThreads), kThreads, 0, s>>>(nbr, indptr, indices,
                                                                           values, x, y);
      });
    else
      k_bsr_spmv<V><<<fv_blocks(rows, kThreads), kThreads, 0, s>>>(nbr, b, indptr, indices,
                                                                   values, x, y);
    FV_CUDA_TRY(cudaGetLastError());
    return FV_OK;
  }
  // transposed product: build the transpose map of the (device) pattern on the host once per call
  std::vector<int> hp(nbr + 1);
  FV_CUDA_TRY(cudaMemcpyAsync(hp.data(), indptr, sizeof(int) * (nbr + 1), cudaMemcpyDeviceToHost, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < nbr; ++i)
    if (hp[i] > hp[i + 1] || hp[0] != 0) {
      fv_set_error("fv_bsr_spmv: indptr is not a non-decreasing offset list from 0");
      return FV_ERR_ARG;
    }
  std::vector<int> hi(hp[nbr]);
  FV_CUDA_TRY(cudaMemcpy(hi.data(), indices, sizeof(int) * hp[nbr], cudaMemcpyDeviceToHost));
  for (int q = 0; q < hp[nbr]; ++q)
    if (hi[q] < 0 || hi[q] >= nbr) {
      fv_set_error("fv_bsr_spmv: column index %d at block %d out of range [0, %d)", hi[q], q, nbr);
      return FV_ERR_ARG;
    }
  Transpose T;
  build_transpose(nbr, nbr, hp.data(), hi.data(), &T);
  int *tp = nullptr, *ti = nullptr, *tb = nullptr;
  if (upload(T.ptr, &tp, s) || upload(T.idx, &ti, s) || upload(T.blk, &tb, s)) {
    cudaFree(tp);
    cudaFree(ti);
    cudaFree(tb);
    return FV_ERR_CUDA;
  }
  launch_spmv_t<V>(nbr, b, tp, ti, tb, values, x, y, s);
  FV_CUDA_TRY(cudaGetLastError());
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  cudaFree(tp);
  cudaFree(ti);
  cudaFree(tb);
  return FV_OK;
}
}  // namespace

// Transpose map of a square BSR pattern (host): for block row j of A^T the rows i of A with a
// block (i, j) (tptr / tidx) and that block's index in A (tblk).  tptr n + 1; tidx, tblk nnzb.
extern "C" int fv_bsr_transpose_map(int n, const int* indptr, const int* indices, int* tptr,
                                    int* tidx, int* tblk) {
  if (n <= 0 || !indptr || !indices || !tptr || !tidx || !tblk) {
    fv_set_error("fv_bsr_transpose_map: bad arguments");
    return FV_ERR_ARG;
  }
  if (!fv_offsets_ok("fv_bsr_transpose_map", n, indptr)) return FV_ERR_ARG;
  for (int q = 0; q < indptr[n]; ++q)
    if (indices[q] < 0 || indices[q] >= n) {
      fv_set_error("fv_bsr_transpose_map: column index out of range");
      return FV_ERR_ARG;
    }
  Transpose T;
  build_transpose(n, n, indptr, indices, &T);
  std::copy(T.ptr.begin(), T.ptr.end(), tptr);
  std::copy(T.idx.begin(), T.idx.end(), tidx);
  std::copy(T.blk.begin(), T.blk.end(), tblk);
  return FV_OK;
}

// y = A^T x through a transpose map from fv_bsr_transpose_map (device arrays; no allocation).
extern "C" int fv_bsr_spmv_t_mapped(int n, int b, const int* tptr, const int* tidx,
                                    const int* tblk, const void* values, const void* x, void* y,
                                    int f64, void* stream) {
  if (n <= 0 || b <= 0 || !tptr || !tidx || !tblk || !values || !x || !y) {
    fv_set_error("fv_bsr_spmv_t_mapped: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (f64)
    launch_spmv_t<double>(n, b, tptr, tidx, tblk, (const double*)values, (const double*)x,
                          (double*)y, s);
  else
    launch_spmv_t<float>(n, b, tptr, tidx, tblk, (const float*)values, (const float*)x, (float*)y,
                         s);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_bsr_transpose_blocks(long nnzb, int b, const int* tblk, const void* values,
                                       void* tvalues, int f64, void* stream) {
  if (nnzb <= 0 || b <= 0 || !tblk || !values || !tvalues) {
    fv_set_error("fv_bsr_transpose_blocks: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  const long nv = nnzb * b * b;
  if (f64)
    k_transpose_blocks<double><<<fv_blocks(nv, kThreads), kThreads, 0, s>>>(
        nnzb, b, tblk, (const double*)values, (double*)tvalues);
  else
    k_transpose_blocks<float><<<fv_blocks(nv, kThreads), kThreads, 0, s>>>(
        nnzb, b, tblk, (const float*)values, (float*)tvalues);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_bsr_spmv_f64(int nbr, int b, const int* indptr, const int* indices,
                               const double* values, const double* x, double* y, int transpose,
                               void* stream) {
  return spmv<double>(nbr, b, indptr, indices, values, x, y, transpose, (cudaStream_t)stream);
}
extern "C" int fv_bsr_spmv_f32(int nbr, int b, const int* indptr, const int* indices,
                               const float* values, const float* x, float* y, int transpose,
                               void* stream) {
  return spmv<float>(nbr, b, indptr, indices, values, x, y, transpose, (cudaStream_t)stream);
}

// out[i] = sum over fields q and cells c in [seg[i], seg[i + 1]) of a[q nc + c] b[q nc + c]: one
// block per segment, fixed summation order.
__global__ void k_segment_dot(const int* seg, int nfld, int nc, const double* a, const double* b,
                              double* out) {
  __shared__ double red[256];
  const int i = blockIdx.x;
  const int lo = seg[i], hi = seg[i + 1];
  double acc = 0.0;
  for (int q = 0; q < nfld; ++q)
    for (int c = lo + threadIdx.x; c < hi; c += blockDim.x)
      acc += a[(long)q * nc + c] * b[(long)q * nc + c];
  red[threadIdx.x] = acc;
  __syncthreads();
  for (int h = 128; h > 0; h >>= 1) {
    if (threadIdx.x < h) red[threadIdx.x] += red[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[i] = red[0];
}

extern "C" int fv_segment_dot(int n_seg, const int* seg, int nfld, int nc, const double* a,
                              const double* b, double* out, void* stream) {
  if (n_seg <= 0 || nfld <= 0 || nc <= 0 || !seg || !a || !b || !out) {
    fv_set_error("fv_segment_dot: bad arguments");
    return FV_ERR_ARG;
  }
  k_segment_dot<<<n_seg, 256, 0, (cudaStream_t)stream>>>(seg, nfld, nc, a, b, out);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_dot_f64(long n, const double* x, const double* y, double* out, void* stream) {
  if (n < 0 || !x || !y || !out) {
    fv_set_error("fv_dot_f64: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (!g_dot_parts) FV_CUDA_TRY(cudaMalloc(&g_dot_parts, sizeof(double) * kRedBlocks));
  k_dot_partial<<<kRedBlocks, kThreads, 0, s>>>(n, x, y, g_dot_parts);
  k_dot_final<<<1, kThreads, 0, s>>>(kRedBlocks, g_dot_parts, out);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}
