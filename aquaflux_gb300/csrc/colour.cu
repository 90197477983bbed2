// Saturation-degree greedy colouring of a conflict graph (host code).
//
// Restates the bucket-queue algorithm of aquaflux/solve/sparse_jacobian.py:409-534
// (_saturation_colouring) so that the colours are identical to the reference's for the same
// conflict graph (same CSR neighbour order):
//   * rank(v) = saturation(v) * (max_degree + 1) + degree(v); vertices sit in one bucket per
//     rank, each bucket a doubly linked list with insertion at the head;
//   * initially every vertex is inserted in index order into the bucket of its degree;
//   * each step takes the head of the highest non-empty bucket, gives it the smallest colour not
//     taken by a coloured neighbour, then, for every still-uncoloured neighbour (in CSR order)
//     seeing that colour for the first time, moves it to the head of its new (higher) bucket.
// Runs in O(n + m) with a bitset of taken colours per vertex.
#include <algorithm>
#include <cstdint>
#include <memory>
#include <vector>

#include "host_par.h"
#include "internal.cuh"

extern "C" int fv_saturation_colouring(int n, const int* indptr, const int* indices, int* colour,
                                       int* n_colours) {
  if (n < 0 || (n > 0 && (!indptr || !indices || !colour))) {
    fv_set_error("fv_saturation_colouring: bad arguments");
    return FV_ERR_ARG;
  }
  if (n == 0) {
    if (n_colours) *n_colours = 0;
    return FV_OK;
  }
  if (!fv_offsets_ok("fv_saturation_colouring", n, indptr)) return FV_ERR_ARG;
  long max_degree = 0;
  for (int v = 0; v < n; ++v) max_degree = std::max<long>(max_degree, indptr[v + 1] - indptr[v]);
  for (long q = 0; q < indptr[n]; ++q)
    if (indices[q] < 0 || indices[q] >= n) {
      fv_set_error("fv_saturation_colouring: neighbour index out of range");
      return FV_ERR_ARG;
    }
  const long words = max_degree / 64 + 2;
  const long tie = max_degree + 1;
  // per vertex: its bucket rank and its links in the bucket's list (one cache line holds four)
  struct Node {
    long rank;
    int next, prev;
  };
  std::vector<Node> node(n);
  std::vector<uint64_t> taken((size_t)n * words, 0);
  std::vector<int> head((size_t)(tie * max_degree + max_degree + 1), -1);
  for (int v = 0; v < n; ++v) colour[v] = -1;
  long top = 0;
  for (int v = 0; v < n; ++v) {
    const long r = indptr[v + 1] - indptr[v];
    const int h = head[r];
    node[v] = Node{r, h, -1};
    if (h >= 0) node[h].prev = v;
    head[r] = v;
    top = std::max(top, r);
  }
  int ncol = 0;
  for (int step = 0; step < n; ++step) {
    while (head[top] < 0) --top;
    const int v = head[top];
    const int f = node[v].next;
    head[top] = f;
    if (f >= 0) node[f].prev = -1;
    int chosen = -1;
    for (long w = 0; w < words; ++w) {
      const uint64_t freeb = ~taken[(size_t)v * words + w];
      if (freeb) {
        chosen = (int)(w * 64 + __builtin_ctzll(freeb));
        break;
      }
    }
    colour[v] = chosen;
    ncol = std::max(ncol, chosen + 1);
    const long word = chosen / 64;
    const uint64_t bit = 1ull << (chosen % 64);
    // every uncoloured neighbour seeing the colour for the first time moves, in CSR order, to the
    // head of the bucket one saturation higher (a coloured neighbour's bits are never read again)
    for (int q = indptr[v]; q < indptr[v + 1]; ++q) {
      const int u = indices[q];
      if (colour[u] >= 0) continue;
      uint64_t& t = taken[(size_t)u * words + word];
      if (t & bit) continue;
      t |= bit;
      Node& nu = node[u];
      const long r_old = nu.rank, r_new = r_old + tie;
      if (nu.prev >= 0) node[nu.prev].next = nu.next;
      else head[r_old] = nu.next;
      if (nu.next >= 0) node[nu.next].prev = nu.prev;
      const int h = head[r_new];
      nu.rank = r_new;
      nu.next = h;
      nu.prev = -1;
      if (h >= 0) node[h].prev = u;
      head[r_new] = u;
      top = std::max(top, r_new);
    }
  }
  if (n_colours) *n_colours = ncol;
  return FV_OK;
}

// First-fit greedy colouring in index order (every vertex takes the smallest colour none of its
// already coloured neighbours has): O(edges), for orderings where the colour count matters more
// than its minimality (the AMG fine smoother's red-black-like sweeps).
extern "C" int fv_greedy_colouring(int n, const int* indptr, const int* indices, int* colour,
                                   int* n_colours) {
  if (n < 0 || (n > 0 && (!indptr || !indices || !colour))) {
    fv_set_error("fv_greedy_colouring: bad arguments");
    return FV_ERR_ARG;
  }
  if (n > 0 && !fv_offsets_ok("fv_greedy_colouring", n, indptr)) return FV_ERR_ARG;
  int ncol = 0;
  std::vector<int> seen(64, -1);
  for (int v = 0; v < n; ++v) colour[v] = -1;
  for (int v = 0; v < n; ++v) {
    for (int q = indptr[v]; q < indptr[v + 1]; ++q) {
      const int u = indices[q];
      if (u < 0 || u >= n) {
        fv_set_error("fv_greedy_colouring: neighbour index out of range");
        return FV_ERR_ARG;
      }
      const int c = colour[u];
      if (c >= 0) {
        if (c >= (int)seen.size()) seen.resize(2 * c + 2, -1);
        seen[c] = v;
      }
    }
    int c = 0;
    while (c < (int)seen.size() && seen[c] == v) ++c;
    colour[v] = c;
    if (c + 1 > ncol) ncol = c + 1;
  }
  if (n_colours) *n_colours = ncol;
  return FV_OK;
}

// Reach-1 cell pattern (host): row i holds i and the cells sharing a face with i, sorted and
// unique.  Interior faces given as (owner, neighbour) pairs.  indptr (n + 1); indices receives
// at most n + 2 * n_pairs entries.
extern "C" int fv_cell_pattern(int n, long n_pairs, const int* owner, const int* neighbour,
                               int* indptr, int* indices) {
  if (n <= 0 || n_pairs < 0 || (n_pairs > 0 && (!owner || !neighbour)) || !indptr || !indices) {
    fv_set_error("fv_cell_pattern: bad arguments");
    return FV_ERR_ARG;
  }
  // 1. every pair chunk counts its two entries (row a: b, row b: a) per destination row range
  const HostSplit rows = host_split(n, 1 << 16), pairs = host_split(n_pairs, 1 << 16);
  const long R = rows.nt, P = pairs.nt;
  std::vector<long> count((size_t)P * R, 0);  // [pair chunk][row range]
  std::vector<long> bad(P, -1);
  host_parallel_for(n_pairs, 1 << 16, [&](long f0, long f1, int t) {
    long* c = count.data() + (size_t)t * R;
    for (long f = f0; f < f1; ++f) {
      const int a = owner[f], b = neighbour[f];
      if (a < 0 || a >= n || b < 0 || b >= n) {
        bad[t] = f;
        return;
      }
      ++c[a / rows.chunk];
      ++c[b / rows.chunk];
    }
  });
  for (long t = 0; t < P; ++t)
    if (bad[t] >= 0) {
      fv_set_error("fv_cell_pattern: cell index out of range at pair %ld", bad[t]);
      return FV_ERR_ARG;
    }
  // 2. bucket the entries by row range (range-major, pair chunks in order within a range)
  std::vector<long> off((size_t)P * R + 1, 0), range_start(R + 1, 0);
  {
    long pos = 0;
    for (long k = 0; k < R; ++k) {
      range_start[k] = pos;
      for (long t = 0; t < P; ++t) {
        off[(size_t)t * R + k] = pos;
        pos += count[(size_t)t * R + k];
      }
    }
    range_start[R] = pos;
  }
  // scratch without value-initialisation: the threads below touch it first, in parallel
  std::unique_ptr<int2[]> ent(new int2[std::max(1L, range_start[R])]);
  host_parallel_for(n_pairs, 1 << 16, [&](long f0, long f1, int t) {
    long* o = off.data() + (size_t)t * R;
    for (long f = f0; f < f1; ++f) {
      const int a = owner[f], b = neighbour[f];
      ent[o[a / rows.chunk]++] = make_int2(a, b);
      ent[o[b / rows.chunk]++] = make_int2(b, a);
    }
  });
  // 3. each row range fills, sorts and de-duplicates its own rows (the diagonal included); a
  // range's rows start after the previous ranges' entries and diagonals, and every per-row
  // array element is written by the range owning the row only
  std::vector<long> start(n);
  std::vector<int> deg(n, 1), width(n);
  std::unique_ptr<int[]> tmp(new int[range_start[R] + n]);
  host_parallel_for(n, 1 << 16, [&](long r0, long r1, int k) {
    for (long e = range_start[k]; e < range_start[k + 1]; ++e) ++deg[ent[e].x];
    long pos = range_start[k] + r0;
    for (long i = r0; i < r1; ++i) {
      start[i] = pos;
      pos += deg[i];
    }
    std::vector<long> fill(start.begin() + r0, start.begin() + r1);
    for (long i = r0; i < r1; ++i) tmp[fill[i - r0]++] = (int)i;
    for (long e = range_start[k]; e < range_start[k + 1]; ++e)
      tmp[fill[ent[e].x - r0]++] = ent[e].y;
    for (long i = r0; i < r1; ++i) {
      int* b = tmp.get() + start[i];
      int* e = b + deg[i];
      std::sort(b, e);
      width[i] = (int)(std::unique(b, e) - b);
    }
  });
  long pos = 0;
  indptr[0] = 0;
  for (int i = 0; i < n; ++i) {
    pos += width[i];
    if (pos > 0x7fffffffL) {
      fv_set_error("fv_cell_pattern: pattern exceeds int32 entries");
      return FV_ERR_ARG;
    }
    indptr[i + 1] = (int)pos;
  }
  host_parallel_for(n, 1 << 16, [&](long r0, long r1, int) {
    for (long i = r0; i < r1; ++i)
      std::copy(tmp.get() + start[i], tmp.get() + start[i] + width[i], indices + indptr[i]);
  });
  return FV_OK;
}
