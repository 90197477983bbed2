/* CPU oracle of zero-fill ILU(0) -- TEST INFRASTRUCTURE ONLY (never linked by the product).
 *
 * Plain-C restatement of the reference's compiled kernel aquaflux/solve/_ilu0.pyx:
 *   ilu0_diagonal_positions  <- diagonal_positions  (:35-65)
 *   ilu0_factor              <- factor              (:68-121)   IKJ, in place, O(1) position map
 *   ilu0_solve               <- solve               (:124-147)  forward then backward sweep
 *   ilu0_solve_transpose     <- solve_transpose     (:150-178)  scatter-form U^T then L^T
 * Return codes: 0 ok, 3 missing diagonal (row in *bad), 4 zero pivot (pivot row in *bad).
 * Compiled without FMA contraction so it rounds exactly like the reference.
 */
#include <stdlib.h>

int ilu0_diagonal_positions(const int *indptr, const int *indices, int n, int *diag, int *bad) {
  for (int i = 0; i < n; ++i) {
    int found = -1;
    for (int q = indptr[i]; q < indptr[i + 1]; ++q)
      if (indices[q] == i) { found = q; break; }
    if (found < 0) { *bad = i; return 3; }
    diag[i] = found;
  }
  return 0;
}

int ilu0_factor(const int *indptr, const int *indices, double *data, const int *diag, int n,
                int *bad) {
  int *position = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  if (!position) return 1;
  for (int i = 0; i < n; ++i) position[i] = -1;
  int rc = 0;
  for (int i = 0; i < n && rc == 0; ++i) {
    for (int q = indptr[i]; q < indptr[i + 1]; ++q) position[indices[q]] = q;
    for (int q = indptr[i]; q < indptr[i + 1]; ++q) {
      int j = indices[q];
      if (j >= i) break;
      double pivot = data[diag[j]];
      if (pivot == 0.0) { *bad = j; rc = 4; break; }
      data[q] = data[q] / pivot;
      double f = data[q];
      for (int q2 = diag[j] + 1; q2 < indptr[j + 1]; ++q2) {
        int slot = position[indices[q2]];
        if (slot != -1) data[slot] = data[slot] - f * data[q2];
      }
    }
    for (int q = indptr[i]; q < indptr[i + 1]; ++q) position[indices[q]] = -1;
  }
  free(position);
  return rc;
}

void ilu0_solve(const int *indptr, const int *indices, const double *data, const int *diag,
                double *x, int n) {
  for (int i = 0; i < n; ++i) {
    double acc = x[i];
    for (int q = indptr[i]; q < diag[i]; ++q) acc = acc - data[q] * x[indices[q]];
    x[i] = acc;
  }
  for (int i = n - 1; i >= 0; --i) {
    double acc = x[i];
    for (int q = diag[i] + 1; q < indptr[i + 1]; ++q) acc = acc - data[q] * x[indices[q]];
    x[i] = acc / data[diag[i]];
  }
}

void ilu0_solve_transpose(const int *indptr, const int *indices, const double *data,
                          const int *diag, double *x, int n) {
  for (int i = 0; i < n; ++i) {
    double v = x[i] / data[diag[i]];
    x[i] = v;
    for (int q = diag[i] + 1; q < indptr[i + 1]; ++q) x[indices[q]] = x[indices[q]] - data[q] * v;
  }
  for (int i = n - 1; i >= 0; --i) {
    double v = x[i];
    for (int q = indptr[i]; q < diag[i]; ++q) x[indices[q]] = x[indices[q]] - data[q] * v;
  }
}
