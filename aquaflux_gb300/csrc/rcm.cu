// Cell graph and reverse Cuthill-McKee renumbering on the GPU.
//
// The reference relabels cells with ReverseCuthillMcKee (aquaflux/mesh/reorder.py:147-159):
// scipy.sparse.csgraph.reverse_cuthill_mckee(symmetric_mode=True) on the cell adjacency of the
// interior faces (cell_adjacency_coo, aquaflux/mesh/graph.py:29-56, coalesced to a sorted CSR).
// The permutation must be bit-identical, so this restates scipy's published algorithm exactly:
//   * seeds are taken in the order of numpy's argsort of the node degrees (the caller passes that
//     order, computed by the same numpy call on the host), skipping placed nodes -- one
//     breadth-first sweep per connected component;
//   * a sweep processes the current level's nodes in their placement order; each appends its
//     not-yet-placed neighbours, then sorts just those by degree with a stable insertion sort
//     (neighbours are visited in ascending index order, so the key is (degree, index));
//   * the Cuthill-McKee order is reversed at the end.
// A node adjacent to several nodes of a level is appended by the first of them in placement
// order.  Level-parallel form: every level's parents claim their unplaced neighbours with an
// atomicMin of the parent's position (placed nodes hold -1, below any position, so they are never
// claimed), each parent then collects the neighbours it won, sorts them, and writes them at its
// exclusive-scan offset -- exactly the sequential order.  One host round trip per level (its size).
#include <algorithm>
#include <climits>
#include <vector>

#include "internal.cuh"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxDegree = 64;  // per-node neighbour bound of the parent-local sort

__global__ void k_fill_int(long n, int* a, int v) {
  long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] = v;
}

// cnt[c + 1] += 1 for both cells of every interior pair (pairs outside [0, n) are skipped and
// flagged)
__global__ void k_graph_count(long np, int n, const int* own, const int* nb, int* cnt, int* bad) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int a = own[p], b = nb[p];
  if (a < 0 || a >= n || b < 0 || b >= n || a == b) {
    atomicExch(bad, 1);
    return;
  }
  atomicAdd(&cnt[a + 1], 1);
  atomicAdd(&cnt[b + 1], 1);
}

// In-place inclusive scan of a[0..n) by one block of 1024 threads (contiguous chunk per thread,
// then the chunk totals); *total (optional) receives a[n - 1].
__global__ void k_scan(long n, int* a, int* total) {
  __shared__ int tot[1024];
  const int t = threadIdx.x, nt = blockDim.x;
  const long chunk = (n + nt - 1) / nt;
  const long b0 = (long)t * chunk, b = b0 < n ? b0 : n;
  const long e = b + chunk < n ? b + chunk : n;
  int s = 0;
  for (long i = b; i < e; ++i) {
    s += a[i];
    a[i] = s;
  }
  tot[t] = s;
  __syncthreads();
  if (t == 0)
    for (int k = 1; k < nt; ++k) tot[k] += tot[k - 1];
  __syncthreads();
  const int off = t > 0 ? tot[t - 1] : 0;
  for (long i = b; i < e; ++i) a[i] += off;
  if (total && t == nt - 1) *total = tot[nt - 1];
}

__global__ void k_graph_fill(long np, const int* own, const int* nb, const int* ptr0, int* cursor,
                             int* tmp) {
  long p = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const int a = own[p], b = nb[p];
  tmp[ptr0[a] + atomicAdd(&cursor[a], 1)] = b;
  tmp[ptr0[b] + atomicAdd(&cursor[b], 1)] = a;
}

// Sort each row's neighbours ascending (insertion sort) and count the distinct ones.
__global__ void k_graph_sort(int n, const int* ptr0, int* tmp, int* ucnt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int b = ptr0[i], e = ptr0[i + 1];
  for (int p = b + 1; p < e; ++p) {
    const int v = tmp[p];
    int q = p - 1;
    while (q >= b && tmp[q] > v) {
      tmp[q + 1] = tmp[q];
      --q;
    }
    tmp[q + 1] = v;
  }
  int u = 0;
  for (int p = b; p < e; ++p) u += (p == b || tmp[p] != tmp[p - 1]) ? 1 : 0;
  ucnt[i + 1] = u;
}

__global__ void k_graph_compact(int n, const int* ptr0, const int* tmp, const int* ptr, int* idx) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int w = ptr[i];
  for (int p = ptr0[i]; p < ptr0[i + 1]; ++p)
    if (p == ptr0[i] || tmp[p] != tmp[p - 1]) idx[w++] = tmp[p];
}

// Level [ls, le) of order: every parent claims its unplaced neighbours.
__global__ void k_rcm_claim(int ls, int le, const int* order, const int* ptr, const int* idx,
                            int* mark) {
  const int p = ls + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= le) return;
  const int i = order[p];
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) atomicMin(&mark[idx[q]], p);
}

// cnt[p - ls] = neighbours parent p won.
__global__ void k_rcm_count(int ls, int le, const int* order, const int* ptr, const int* idx,
                            const int* mark, int* cnt) {
  const int p = ls + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= le) return;
  const int i = order[p];
  int c = 0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) c += mark[idx[q]] == p ? 1 : 0;
  cnt[p - ls] = c;
}

// Parent p writes the neighbours it won, sorted by (degree, index), after its inclusive-scan
// predecessor's, and marks them placed.
__global__ void k_rcm_place(int ls, int le, int* order, const int* ptr, const int* idx,
                            int* mark, const int* incl) {
  const int p = ls + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= le) return;
  const int i = order[p];
  int kid[kMaxDegree], kdeg[kMaxDegree];
  int c = 0;
  for (int q = ptr[i]; q < ptr[i + 1]; ++q) {
    const int j = idx[q];
    if (mark[j] != p) continue;
    const int d = ptr[j + 1] - ptr[j];
    int t = c++;
    while (t > 0 && d < kdeg[t - 1]) {  // stable: equal degrees keep ascending index order
      kid[t] = kid[t - 1];
      kdeg[t] = kdeg[t - 1];
      --t;
    }
    kid[t] = j;
    kdeg[t] = d;
  }
  const int base = le + (p > ls ? incl[p - ls - 1] : 0);
  for (int t = 0; t < c; ++t) {
    order[base + t] = kid[t];
    mark[kid[t]] = -1;
  }
}

__global__ void k_rcm_perm(int n, const int* order, int* perm) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) perm[order[k]] = n - 1 - k;
}

__global__ void k_set(int* a, int i, int v) { a[i] = v; }

int blocks_of(long n) { return (int)std::max(1L, (n + kThreads - 1) / kThreads); }

}  // namespace

extern "C" int fv_cell_graph(int n, long n_pairs, const int* owner, const int* neighbour,
                             int* indptr, int* indices, int* work, void* stream) {
  if (n <= 0 || n_pairs < 0 || !indptr || !work || (n_pairs > 0 && (!owner || !neighbour || !indices))) {
    fv_set_error("fv_cell_graph: bad arguments");
    return FV_ERR_ARG;
  }
  if (2 * n_pairs > INT_MAX) {
    fv_set_error("fv_cell_graph: too many pairs for int32 offsets");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  int* ptr0 = work;                 // n + 1
  int* cursor = ptr0 + n + 1;       // n
  int* bad = cursor + n;            // 1
  int* tmp = bad + 1;               // 2 n_pairs
  k_fill_int<<<blocks_of(2L * n + 2), kThreads, 0, s>>>(2L * n + 2, ptr0, 0);
  k_fill_int<<<blocks_of(n + 1), kThreads, 0, s>>>(n + 1, indptr, 0);
  if (n_pairs > 0) {
    k_graph_count<<<blocks_of(n_pairs), kThreads, 0, s>>>(n_pairs, n, owner, neighbour, ptr0, bad);
    int h_bad = 0;
    FV_CUDA_TRY(cudaMemcpyAsync(&h_bad, bad, sizeof(int), cudaMemcpyDeviceToHost, s));
    FV_CUDA_TRY(cudaStreamSynchronize(s));
    if (h_bad) {
      fv_set_error("fv_cell_graph: a cell pair is out of range or joins a cell to itself");
      return FV_ERR_ARG;
    }
    k_scan<<<1, 1024, 0, s>>>(n + 1, ptr0, nullptr);
    k_graph_fill<<<blocks_of(n_pairs), kThreads, 0, s>>>(n_pairs, owner, neighbour, ptr0, cursor,
                                                         tmp);
    k_graph_sort<<<blocks_of(n), kThreads, 0, s>>>(n, ptr0, tmp, indptr);
    k_scan<<<1, 1024, 0, s>>>(n + 1, indptr, nullptr);
    k_graph_compact<<<blocks_of(n), kThreads, 0, s>>>(n, ptr0, tmp, indptr, indices);
  }
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_rcm_permutation(int n, const int* indptr, const int* indices,
                                  const long* seed_order, int* perm, int* work, void* stream) {
  if (n <= 0 || !indptr || !seed_order || !perm || !work) {
    fv_set_error("fv_rcm_permutation: bad arguments");
    return FV_ERR_ARG;
  }
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<int> hptr(n + 1);
  FV_CUDA_TRY(cudaMemcpyAsync(hptr.data(), indptr, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s));
  FV_CUDA_TRY(cudaStreamSynchronize(s));
  for (int i = 0; i < n; ++i)
    if (hptr[i + 1] - hptr[i] > kMaxDegree || hptr[i + 1] < hptr[i]) {
      fv_set_error("fv_rcm_permutation: node %d has degree %d (at most %d)", i,
                   hptr[i + 1] - hptr[i], kMaxDegree);
      return FV_ERR_ARG;
    }
  int* order = work;        // n
  int* mark = order + n;    // n: -1 placed, INT_MAX unclaimed, else the claiming position
  int* cnt = mark + n;      // n: per-parent counts of a level, scanned in place
  int* total = cnt + n;     // 1
  k_fill_int<<<blocks_of(n), kThreads, 0, s>>>(n, mark, INT_MAX);
  std::vector<char> placed(n, 0);
  std::vector<int> seg;
  int n_placed = 0;
  long next = 0;  // position in seed_order
  while (n_placed < n) {
    while (next < n && placed[seed_order[next]]) ++next;
    if (next >= n) {
      fv_set_error("fv_rcm_permutation: seed order is not a permutation");
      return FV_ERR_ARG;
    }
    const int seed = (int)seed_order[next];
    if (seed < 0 || seed >= n) {
      fv_set_error("fv_rcm_permutation: seed %d out of range", seed);
      return FV_ERR_ARG;
    }
    k_set<<<1, 1, 0, s>>>(order, n_placed, seed);
    k_set<<<1, 1, 0, s>>>(mark, seed, -1);
    int ls = n_placed, le = n_placed + 1;
    while (ls < le) {
      const int L = le - ls;
      k_rcm_claim<<<blocks_of(L), kThreads, 0, s>>>(ls, le, order, indptr, indices, mark);
      k_rcm_count<<<blocks_of(L), kThreads, 0, s>>>(ls, le, order, indptr, indices, mark, cnt);
      k_scan<<<1, 1024, 0, s>>>(L, cnt, total);
      k_rcm_place<<<blocks_of(L), kThreads, 0, s>>>(ls, le, order, indptr, indices, mark, cnt);
      int h_total = 0;
      FV_CUDA_TRY(cudaMemcpyAsync(&h_total, total, sizeof(int), cudaMemcpyDeviceToHost, s));
      FV_CUDA_TRY(cudaStreamSynchronize(s));
      if (h_total < 0 || h_total > n - le) {
        fv_set_error("fv_rcm_permutation: inconsistent level size %d", h_total);
        return FV_ERR_ARG;
      }
      ls = le;
      le += h_total;
    }
    // the component just placed: mark it on the host for the next seed search
    seg.resize(le - n_placed);
    FV_CUDA_TRY(cudaMemcpyAsync(seg.data(), order + n_placed, sizeof(int) * seg.size(),
                                cudaMemcpyDeviceToHost, s));
    FV_CUDA_TRY(cudaStreamSynchronize(s));
    for (int v : seg) placed[v] = 1;
    n_placed = le;
  }
  k_rcm_perm<<<blocks_of(n), kThreads, 0, s>>>(n, order, perm);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}
