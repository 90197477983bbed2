// Aggregation multigrid pieces: cell aggregation (host), Galerkin coarse operators, restriction
// and prolongation (device).
//
// The hierarchy follows the reference's aggregation AMG for the coupled block operator
// (aquaflux/solve/multigrid.py:1011-1245 _build_aggregation_hierarchy, :353 _mis_aggregate, used
// by the ILU-smoothed V-cycle of aquaflux/solve/ilu_inverse.py:160-308): cells are aggregated on
// the cell graph, every field of a cell rides its aggregate's coarse unknown (block-size aware),
// and the coarse operator is the Galerkin product P^T A P.  Here P is the unsmoothed (piecewise
// constant) tentative prolongation, so P^T A P is an aggregate-to-aggregate sum of fine blocks: the
// GPU forms each coarse block as the ordered sum of its fine blocks (deterministic, no atomics).
#include <algorithm>
#include <memory>
#include <vector>

#include "host_par.h"
#include "internal.cuh"

// Greedy aggregation of a symmetric cell graph (CSR, self loops ignored):
//   pass 1 -- cells in index order whose whole neighbourhood is free become the root of an
//             aggregate holding the cell and its neighbours;
//   pass 2 -- a free cell joins the aggregate of its first aggregated neighbour;
//   pass 3 -- cells still free group with their free neighbours (or alone).
extern "C" int fv_aggregate(int n, const int* indptr, const int* indices, int* agg, int* n_agg) {
  if (n <= 0 || !indptr || !indices || !agg || !n_agg) {
    fv_set_error("fv_aggregate: bad arguments");
    return FV_ERR_ARG;
  }
  if (!fv_offsets_ok("fv_aggregate", n, indptr)) return FV_ERR_ARG;
  for (int i = 0; i < n; ++i) agg[i] = -1;
  int na = 0;
  for (int i = 0; i < n; ++i) {
    bool free_nb = true;
    for (int q = indptr[i]; q < indptr[i + 1] && free_nb; ++q) {
      const int j = indices[q];
      if (j < 0 || j >= n) {
        fv_set_error("fv_aggregate: neighbour index out of range");
        return FV_ERR_ARG;
      }
      if (agg[j] >= 0) free_nb = false;
    }
    if (!free_nb || agg[i] >= 0) continue;
    agg[i] = na;
    for (int q = indptr[i]; q < indptr[i + 1]; ++q) agg[indices[q]] = na;
    ++na;
  }
  std::vector<int> pass2(n, -1);
  for (int i = 0; i < n; ++i) {
    if (agg[i] >= 0) continue;
    for (int q = indptr[i]; q < indptr[i + 1]; ++q) {
      const int j = indices[q];
      if (j != i && agg[j] >= 0) {
        pass2[i] = agg[j];
        break;
      }
    }
  }
  for (int i = 0; i < n; ++i)
    if (agg[i] < 0 && pass2[i] >= 0) agg[i] = pass2[i];
  for (int i = 0; i < n; ++i) {
    if (agg[i] >= 0) continue;
    agg[i] = na;
    for (int q = indptr[i]; q < indptr[i + 1]; ++q)
      if (agg[indices[q]] < 0) agg[indices[q]] = na;
    ++na;
  }
  *n_agg = na;
  return FV_OK;
}

// First-fit greedy colouring of the aggregates (aggregate graph: two aggregates adjacent when a
// fine block couples their cells), aggregates in index order, read straight from the fine
// pattern: the colour numbering of the coarse levels without forming the coarse pattern first.
extern "C" int fv_colour_aggregates(int n, const int* indptr, const int* indices, const int* agg,
                                    int na, int* colour, int* n_colours) {
  if (n <= 0 || na <= 0 || !indptr || !indices || !agg || !colour) {
    fv_set_error("fv_colour_aggregates: bad arguments");
    return FV_ERR_ARG;
  }
  if (!fv_offsets_ok("fv_colour_aggregates", n, indptr)) return FV_ERR_ARG;
  std::vector<int> cnt(na + 1, 0), members(n);
  for (int i = 0; i < n; ++i) {
    if (agg[i] < 0 || agg[i] >= na) {
      fv_set_error("fv_colour_aggregates: aggregate index out of range at cell %d", i);
      return FV_ERR_ARG;
    }
    ++cnt[agg[i] + 1];
  }
  for (int a = 0; a < na; ++a) cnt[a + 1] += cnt[a];
  {
    std::vector<int> fill(cnt.begin(), cnt.end() - 1);
    for (int i = 0; i < n; ++i) members[fill[agg[i]]++] = i;
  }
  if (host_any_outside(indices, indptr[n], 0, n)) {
    fv_set_error("fv_colour_aggregates: column index out of range");
    return FV_ERR_ARG;
  }
  // the aggregate graph: per aggregate the sorted distinct aggregates its members touch
  // (itself included), i.e. the coarse pattern, built without the block lists; aggregates are
  // split into contiguous ranges over the host threads, each range's rows gathered by its thread
  const long chunk_min = 4096;
  std::vector<std::vector<int>> part(host_threads());
  std::vector<int> len(na, 0);
  host_parallel_for(na, chunk_min, [&](long a0, long a1, int t) {
    std::vector<int> mark(na, -1), row;
    std::vector<int>& out = part[t];
    for (long a = a0; a < a1; ++a) {
      row.clear();
      for (int m = cnt[a]; m < cnt[a + 1]; ++m) {
        const int i = members[m];
        for (int q = indptr[i]; q < indptr[i + 1]; ++q) {
          const int b = agg[indices[q]];
          if (mark[b] != (int)a) {
            mark[b] = (int)a;
            row.push_back(b);
          }
        }
      }
      std::sort(row.begin(), row.end());
      out.insert(out.end(), row.begin(), row.end());
      len[a] = (int)row.size();
    }
  });
  std::vector<int> cptr(na + 1, 0);
  for (int a = 0; a < na; ++a) cptr[a + 1] = cptr[a] + len[a];
  std::vector<int> cidx(cptr[na]);
  host_parallel_for(na, chunk_min, [&](long a0, long, int t) {  // the same split as above
    std::copy(part[t].begin(), part[t].end(), cidx.begin() + cptr[a0]);
  });
  return fv_saturation_colouring(na, cptr.data(), cidx.data(), colour, n_colours);
}

// One coarsening step of a block pattern by an aggregation (host): members of every aggregate
// (ascending fine index), the sorted coarse pattern, and for every coarse block the fine blocks
// that sum into it (ascending fine block index), i.e. the Galerkin product of the piecewise-
// constant prolongation expressed as ordered block lists.
extern "C" int fv_coarsen(int n, const int* indptr, const int* indices, const int* agg, int na,
                          int* mptr, int* mlist, int* cip, int* cix, long* gptr, long* glist,
                          long* n_coarse_blocks) {
  if (n <= 0 || na <= 0 || !indptr || !indices || !agg || !mptr || !mlist || !cip || !cix ||
      !n_coarse_blocks || (!gptr) != (!glist)) {
    fv_set_error("fv_coarsen: bad arguments");
    return FV_ERR_ARG;
  }
  if (!fv_offsets_ok("fv_coarsen", n, indptr)) return FV_ERR_ARG;
  const long nnz = indptr[n];
  for (int i = 0; i < n; ++i)
    if (agg[i] < 0 || agg[i] >= na) {
      fv_set_error("fv_coarsen: aggregate index out of range at cell %d", i);
      return FV_ERR_ARG;
    }
  if (host_any_outside(indices, nnz, 0, n)) {
    fv_set_error("fv_coarsen: column index out of range");
    return FV_ERR_ARG;
  }
  // members (counting sort, stable)
  std::vector<int> cnt(na + 1, 0);
  for (int i = 0; i < n; ++i) ++cnt[agg[i] + 1];
  for (int a = 0; a < na; ++a) cnt[a + 1] += cnt[a];
  for (int a = 0; a <= na; ++a) mptr[a] = cnt[a];
  for (int i = 0; i < n; ++i) mlist[cnt[agg[i]]++] = i;
  // coarse rows: sorted unique aggregate columns (a marker per aggregate column avoids sorting the
  // duplicates), computed per aggregate in parallel into a scratch buffer bounded by the
  // aggregate's fine block count; then the row offsets, then the copy.  With lists, the fine
  // blocks of each coarse block are listed in ascending fine block order, aggregate by aggregate:
  // members ascend within an aggregate and blocks ascend within a row, so a per-aggregate
  // counting pass places them without a global sort.
  const bool lists = gptr != nullptr;  // NULL gptr / glist: the coarse pattern only
  std::vector<long> fb(na + 1, 0);     // fine blocks of each aggregate (prefix)
  for (int a = 0; a < na; ++a) {
    long c = 0;
    for (int m = mptr[a]; m < mptr[a + 1]; ++m) c += indptr[mlist[m] + 1] - indptr[mlist[m]];
    fb[a + 1] = fb[a] + c;
  }
  // scratch without value-initialisation: each aggregate's thread writes its part first
  std::unique_ptr<int[]> scratch(new int[std::max(1L, fb[na])]);
  std::vector<int> width(na);
  const int nth = host_threads();
  std::vector<std::vector<int>> marks(nth), slots(nth);
  host_parallel_for(na, 4096, [&](long b, long e, int t) {
    std::vector<int>& mark = marks[t];
    mark.assign(na, -1);
    for (long a = b; a < e; ++a) {
      int* cols = scratch.get() + fb[a];
      int k = 0;
      for (int m = mptr[a]; m < mptr[a + 1]; ++m) {
        const int i = mlist[m];
        for (int q = indptr[i]; q < indptr[i + 1]; ++q) {
          const int col = agg[indices[q]];
          if (mark[col] != (int)a) {
            mark[col] = (int)a;
            cols[k++] = col;
          }
        }
      }
      std::sort(cols, cols + k);
      width[a] = k;
    }
  });
  cip[0] = 0;
  for (int a = 0; a < na; ++a) cip[a + 1] = cip[a] + width[a];
  const long pos = cip[na];
  *n_coarse_blocks = pos;
  if (lists) {
    // coarse block c of aggregate a holds the fine blocks of its members whose column aggregate
    // is cix[c]: their count, then their offsets
    gptr[0] = 0;
  }
  host_parallel_for(na, 4096, [&](long b, long e, int t) {
    std::vector<int>& slot = slots[t];
    if (lists) slot.assign(na, 0);
    std::vector<long> fill;
    for (long a = b; a < e; ++a) {
      const int k = width[a];
      const int* cols = scratch.get() + fb[a];
      for (int c = 0; c < k; ++c) cix[cip[a] + c] = cols[c];
      if (!lists) continue;
      for (int c = 0; c < k; ++c) slot[cols[c]] = c;
      fill.assign(k + 1, 0);
      for (int m = mptr[a]; m < mptr[a + 1]; ++m) {
        const int i = mlist[m];
        for (int q = indptr[i]; q < indptr[i + 1]; ++q) ++fill[slot[agg[indices[q]]] + 1];
      }
      // this aggregate's fine blocks occupy glist[fb[a], fb[a + 1])
      for (int c = 0; c < k; ++c) {
        fill[c + 1] += fill[c];
        gptr[cip[a] + c + 1] = fb[a] + fill[c + 1];
      }
      for (int m = mptr[a]; m < mptr[a + 1]; ++m) {
        const int i = mlist[m];
        for (int q = indptr[i]; q < indptr[i + 1]; ++q)
          glist[fb[a] + fill[slot[agg[indices[q]]]]++] = q;
      }
    }
  });
  return FV_OK;
}

// Symmetric block permutation of a pattern (host): new row r is old row perm[r]; the new pattern
// (out_indptr (n + 1), out_indices (nnz)) is sorted per row, and bmap[q'] is the old block index of
// new block q'.  iperm is perm's inverse.
extern "C" int fv_permute_pattern(int n, const int* indptr, const int* indices, const int* perm,
                                  int* out_indptr, int* out_indices, long* bmap) {
  if (n <= 0 || !indptr || !indices || !perm || !out_indptr || !out_indices || !bmap) {
    fv_set_error("fv_permute_pattern: bad arguments");
    return FV_ERR_ARG;
  }
  if (!fv_offsets_ok("fv_permute_pattern", n, indptr)) return FV_ERR_ARG;
  std::vector<int> iperm(n, -1);
  for (int r = 0; r < n; ++r) {
    if (perm[r] < 0 || perm[r] >= n || iperm[perm[r]] >= 0) {
      fv_set_error("fv_permute_pattern: perm is not a permutation");
      return FV_ERR_ARG;
    }
    iperm[perm[r]] = r;
  }
  // rows keep their widths: offsets first, then the rows in parallel
  out_indptr[0] = 0;
  for (int r = 0; r < n; ++r) out_indptr[r + 1] = out_indptr[r] + (indptr[perm[r] + 1] - indptr[perm[r]]);
  if (host_any_outside(indices, indptr[n], 0, n)) {
    fv_set_error("fv_permute_pattern: column index out of range");
    return FV_ERR_ARG;
  }
  host_parallel_for(n, 1 << 15, [&](long r0, long r1, int) {
    std::vector<std::pair<int, long>> row;
    for (long r = r0; r < r1; ++r) {
      const int i = perm[r];
      row.clear();
      for (int q = indptr[i]; q < indptr[i + 1]; ++q) row.emplace_back(iperm[indices[q]], (long)q);
      std::sort(row.begin(), row.end());
      long pos = out_indptr[r];
      for (const auto& e : row) {
        out_indices[pos] = e.first;
        bmap[pos] = e.second;
        ++pos;
      }
    }
  });
  return FV_OK;
}

namespace {

// dst block q = src block bmap[q] (b x b entries), converted to Out.
template <class In, class Out>
__global__ void k_gather_blocks(long nnzb, int bb, const long* bmap, const In* src, Out* dst) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nnzb * bb) return;
  const long q = t / bb, e = t % bb;
  dst[t] = (Out)src[bmap[q] * bb + e];
}

// Field-major fp64 vector -> cell-major Out vector in the permuted cell order, scaled:
//   out[r * b + a] = in[a * n + perm[r]] * scale[a * n + perm[r]]   (perm / scale NULL: none)
template <class Out>
__global__ void k_to_cells(int n, int b, const int* perm, const double* scale, const double* in,
                           Out* out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * b) return;
  const int r = (int)(t / b), a = (int)(t % b);
  const long k = (long)a * n + (perm ? perm[r] : r);
  out[t] = (Out)(scale ? in[k] * scale[k] : in[k]);
}

// The inverse: out[a * n + perm[r]] = in[r * b + a] * scale[a * n + perm[r]], widened to fp64.
template <class In>
__global__ void k_from_cells(int n, int b, const int* perm, const double* scale, const In* in,
                             double* out) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n * b) return;
  const int r = (int)(t / b), a = (int)(t % b);
  const long k = (long)a * n + (perm ? perm[r] : r);
  out[k] = scale ? (double)in[t] * scale[k] : (double)in[t];
}

}  // namespace

extern "C" int fv_gather_blocks(long nnzb, int b, const long* bmap, const void* src, int src_f64,
                                void* dst, int dst_f64, void* stream) {
  if (nnzb <= 0 || b <= 0 || !bmap || !src || !dst) {
    fv_set_error("fv_gather_blocks: bad arguments");
    return FV_ERR_ARG;
  }
  const long n = nnzb * b * b;
  const int bb = b * b;
  cudaStream_t s = (cudaStream_t)stream;
  const int g = fv_blocks(n, 256);
  if (src_f64 && dst_f64)
    k_gather_blocks<double, double><<<g, 256, 0, s>>>(nnzb, bb, bmap, (const double*)src, (double*)dst);
  else if (src_f64)
    k_gather_blocks<double, float><<<g, 256, 0, s>>>(nnzb, bb, bmap, (const double*)src, (float*)dst);
  else if (dst_f64)
    k_gather_blocks<float, double><<<g, 256, 0, s>>>(nnzb, bb, bmap, (const float*)src, (double*)dst);
  else
    k_gather_blocks<float, float><<<g, 256, 0, s>>>(nnzb, bb, bmap, (const float*)src, (float*)dst);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_to_cells(int n, int b, const int* perm, const double* scale, const double* in,
                           void* out, int out_f64, void* stream) {
  if (n <= 0 || b <= 0 || !in || !out) {
    fv_set_error("fv_to_cells: bad arguments");
    return FV_ERR_ARG;
  }
  const long m = (long)n * b;
  cudaStream_t s = (cudaStream_t)stream;
  if (out_f64)
    k_to_cells<double><<<fv_blocks(m, 256), 256, 0, s>>>(n, b, perm, scale, in, (double*)out);
  else
    k_to_cells<float><<<fv_blocks(m, 256), 256, 0, s>>>(n, b, perm, scale, in, (float*)out);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

extern "C" int fv_from_cells(int n, int b, const int* perm, const double* scale, const void* in,
                             int in_f64, double* out, void* stream) {
  if (n <= 0 || b <= 0 || !in || !out) {
    fv_set_error("fv_from_cells: bad arguments");
    return FV_ERR_ARG;
  }
  const long m = (long)n * b;
  cudaStream_t s = (cudaStream_t)stream;
  if (in_f64)
    k_from_cells<double><<<fv_blocks(m, 256), 256, 0, s>>>(n, b, perm, scale, (const double*)in, out);
  else
    k_from_cells<float><<<fv_blocks(m, 256), 256, 0, s>>>(n, b, perm, scale, (const float*)in, out);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

namespace {

// coarse[Q] = sum over the fine blocks listed for Q (gptr / glist), in list order, accumulated in
// fp64 and stored in Out.
template <class In, class Out>
__global__ void k_galerkin(long n_coarse_blocks, int b, const long* gptr, const long* glist,
                           const In* fine, Out* coarse) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long bb = (long)b * b;
  if (t >= n_coarse_blocks * bb) return;
  const long Q = t / bb, e = t % bb;
  double acc = 0.0;
  for (long p = gptr[Q]; p < gptr[Q + 1]; ++p) acc += (double)fine[glist[p] * bb + e];
  coarse[t] = (Out)acc;
}

// rc[I * b + a] = sum over the member cells i of aggregate I (mptr / mlist) of r[i * b + a]
template <class T>
__global__ void k_restrict(int n_coarse, int b, const int* mptr, const int* mlist, const T* r,
                           T* rc) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n_coarse * b) return;
  const int I = (int)(t / b), a = (int)(t % b);
  T acc = 0;
  for (int p = mptr[I]; p < mptr[I + 1]; ++p) acc += r[(long)mlist[p] * b + a];
  rc[t] = acc;
}

// x[i * b + a] += xc[agg[i] * b + a]
template <class T>
__global__ void k_prolong_add(int n_fine, int b, const int* agg, const T* xc, T* x) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long)n_fine * b) return;
  const int i = (int)(t / b), a = (int)(t % b);
  x[t] += xc[(long)agg[i] * b + a];
}

template <class Out>
int galerkin(const char* name, long n_coarse_blocks, int b, const long* gptr, const long* glist,
             const void* fine, int fine_f64, Out* coarse, void* stream) {
  if (n_coarse_blocks <= 0 || b <= 0 || !gptr || !glist || !fine || !coarse) {
    fv_set_error("%s: bad arguments", name);
    return FV_ERR_ARG;
  }
  const long n = n_coarse_blocks * b * b;
  cudaStream_t s = (cudaStream_t)stream;
  if (fine_f64)
    k_galerkin<double, Out><<<fv_blocks(n, 256), 256, 0, s>>>(n_coarse_blocks, b, gptr, glist,
                                                              (const double*)fine, coarse);
  else
    k_galerkin<float, Out><<<fv_blocks(n, 256), 256, 0, s>>>(n_coarse_blocks, b, gptr, glist,
                                                             (const float*)fine, coarse);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

template <class T>
int restrict_(const char* name, int n_coarse, int b, const int* mptr, const int* mlist,
              const T* r, T* rc, void* stream) {
  if (n_coarse <= 0 || b <= 0 || !mptr || !mlist || !r || !rc) {
    fv_set_error("%s: bad arguments", name);
    return FV_ERR_ARG;
  }
  const long n = (long)n_coarse * b;
  k_restrict<T><<<fv_blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(n_coarse, b, mptr, mlist, r,
                                                                     rc);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

template <class T>
int prolong_add(const char* name, int n_fine, int b, const int* agg, const T* xc, T* x,
                void* stream) {
  if (n_fine <= 0 || b <= 0 || !agg || !xc || !x) {
    fv_set_error("%s: bad arguments", name);
    return FV_ERR_ARG;
  }
  const long n = (long)n_fine * b;
  k_prolong_add<T><<<fv_blocks(n, 256), 256, 0, (cudaStream_t)stream>>>(n_fine, b, agg, xc, x);
  FV_CUDA_TRY(cudaGetLastError());
  return FV_OK;
}

}  // namespace

extern "C" int fv_galerkin_f32(long n_coarse_blocks, int b, const long* gptr, const long* glist,
                               const void* fine, int fine_f64, float* coarse, void* stream) {
  return galerkin("fv_galerkin_f32", n_coarse_blocks, b, gptr, glist, fine, fine_f64, coarse,
                  stream);
}
extern "C" int fv_galerkin_f64(long n_coarse_blocks, int b, const long* gptr, const long* glist,
                               const void* fine, int fine_f64, double* coarse, void* stream) {
  return galerkin("fv_galerkin_f64", n_coarse_blocks, b, gptr, glist, fine, fine_f64, coarse,
                  stream);
}
extern "C" int fv_restrict_f32(int n_coarse, int b, const int* mptr, const int* mlist,
                               const float* r, float* rc, void* stream) {
  return restrict_("fv_restrict_f32", n_coarse, b, mptr, mlist, r, rc, stream);
}
extern "C" int fv_restrict_f64(int n_coarse, int b, const int* mptr, const int* mlist,
                               const double* r, double* rc, void* stream) {
  return restrict_("fv_restrict_f64", n_coarse, b, mptr, mlist, r, rc, stream);
}
extern "C" int fv_prolong_add_f32(int n_fine, int b, const int* agg, const float* xc, float* x,
                                  void* stream) {
  return prolong_add("fv_prolong_add_f32", n_fine, b, agg, xc, x, stream);
}
extern "C" int fv_prolong_add_f64(int n_fine, int b, const int* agg, const double* xc, double* x,
                                  void* stream) {
  return prolong_add("fv_prolong_add_f64", n_fine, b, agg, xc, x, stream);
}
