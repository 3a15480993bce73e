// CPU oracle for the k-means interpolating-point stage (test infrastructure only).
//
// A single-rank restatement of KMeans::KMeansSolver from the reference
// (src/kmeans.cpp), used by the tests and the CPU baseline as the checker of the
// CUDA path.  It is never linked into the product library.
//
// Followed line by line:
//   guess_initial_centroids   src/kmeans.cpp:159-175   (std::mt19937 + std::shuffle)
//   classify_grid_points      src/kmeans.cpp:88-106    (sqrt distance, first minimum)
//   update_centroids          src/kmeans.cpp:108-144   (sequential sums, weight < 1e-8 fatal)
//   map_to_grid               src/kmeans.cpp:146-157   (roles swapped, then sorted)
//   kernel                    src/kmeans.cpp:187-264   (iteration / convergence logic)
//   normed_difference         src/matrix_operations.h:42-57
//
// Parity is defined at one MPI rank: the reference's Allreduce of per-rank partial
// sums changes the summation order for more ranks.  Build with -ffp-contract=off so
// that no fused multiply-add changes the rounding on hosts whose compiler would
// contract by default (aarch64), matching the x86-64 build of the reference.
// An optional OpenMP variant parallelises the classify loop over grid points; the
// result is identical because each point's argmin is independent.

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <random>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

void classify(const double* pts, int64_t npts, const double* cen, int64_t ncen,
              int* out, int nthreads)
{
#ifdef _OPENMP
#pragma omp parallel for schedule(static) num_threads(nthreads) if (nthreads > 1)
#endif
  for (int64_t i = 0; i < npts; i++) {
    double best = 0.0;
    int64_t arg = 0;
    for (int64_t j = 0; j < ncen; j++) {
      double dx = cen[j * 3] - pts[i * 3];
      double dy = cen[j * 3 + 1] - pts[i * 3 + 1];
      double dz = cen[j * 3 + 2] - pts[i * 3 + 2];
      double d = std::sqrt(dx * dx + dy * dy + dz * dz);
      if (j == 0 || d < best) {  // std::min_element keeps the first minimum
        best = d;
        arg = j;
      }
    }
    out[i] = (int)arg;
  }
  (void)nthreads;
}

double normed_difference(const std::vector<double>& a, const std::vector<double>& b)
{
  double max_a = *std::max_element(a.begin(), a.end());
  double min_a = *std::min_element(a.begin(), a.end());
  double abs_max_a = std::max(std::abs(max_a), std::abs(min_a));
  double max_b = *std::max_element(b.begin(), b.end());
  double min_b = *std::min_element(b.begin(), b.end());
  double abs_max_b = std::max(std::abs(max_b), std::abs(min_b));
  double scale = abs_max_a + abs_max_b;
  double diff = 0.0;
  for (size_t i = 0; i < a.size(); i++) {
    double q = (a[i] - b[i]) / scale;
    diff += q * q;
  }
  return scale * std::sqrt(diff);
}

}  // namespace

extern "C" {

// Initial interpolating-point indices: shuffle 0..ng-1 with mt19937(seed), keep the
// first nmu, sort ascending (src/kmeans.cpp:159-168).
int orc_initial_indices(int64_t ng, int nmu, unsigned int seed, int* out_idx)
{
  if (ng <= 0 || nmu <= 0 || nmu > ng) return 1;
  std::vector<int> tmp(ng);
  for (int64_t i = 0; i < ng; i++) tmp[i] = (int)i;
  std::mt19937 mt(seed);
  std::shuffle(tmp.begin(), tmp.end(), mt);
  std::sort(tmp.begin(), tmp.begin() + nmu);
  std::copy(tmp.begin(), tmp.begin() + nmu, out_idx);
  return 0;
}

// Classify ng points against nmu centroids (both N x 3 C order).
void orc_classify(const double* grid, int64_t ng, const double* cen, int nmu, int* labels,
                  int nthreads)
{
  classify(grid, ng, cen, nmu, labels, nthreads);
}

// Full k-means at one rank.
//   status: 0 ok, 2 empty cluster (the reference exits), 3 bad argument.
//   out_idx receives the sorted interpolating indices; out_iters the number of
//   completed iterations; out_diff the last normed difference; out_centroids (nmu x 3)
//   the centroids handed to map_to_grid; out_labels (optional) the last labels;
//   out_diffs / out_pct (optional, max_it each) every iteration's normed difference and
//   percentage_change (src/kmeans.cpp:177-185, :236-237).
int orc_kmeans(const double* grid, const double* rho, int64_t ng, int nmu,
               const int* init_idx, int max_it, double threshold, int nthreads,
               int* out_idx, int* out_iters, double* out_diff, double* out_centroids,
               int* out_labels, double* out_diffs, double* out_pct)
{
  if (ng <= 0 || nmu <= 0 || nmu > ng || max_it < 1) return 3;
  std::vector<double> cur(3 * (size_t)nmu), nxt(3 * (size_t)nmu);
  for (int k = 0; k < nmu; k++)
    for (int d = 0; d < 3; d++) cur[3 * k + d] = grid[3 * (int64_t)init_idx[k] + d];
  std::vector<int> map(ng), old_map(ng);
  std::vector<double> w(nmu);
  classify(grid, ng, cur.data(), nmu, map.data(), nthreads);
  old_map = map;
  double diff = 0.0;
  int it_done = 0;
  bool converged = false;
  for (int it = 0; it < max_it; it++) {
    classify(grid, ng, cur.data(), nmu, map.data(), nthreads);
    std::fill(w.begin(), w.end(), 0.0);
    std::fill(nxt.begin(), nxt.end(), 0.0);
    for (int64_t i = 0; i < ng; i++) {
      int k = map[i];
      w[k] += rho[i];
      nxt[3 * k] += rho[i] * grid[3 * i];
      nxt[3 * k + 1] += rho[i] * grid[3 * i + 1];
      nxt[3 * k + 2] += rho[i] * grid[3 * i + 2];
    }
    bool critical = false;
    for (int k = 0; k < nmu; k++) {
      if (w[k] < 1e-8) critical = true;
      nxt[3 * k] /= w[k];
      nxt[3 * k + 1] /= w[k];
      nxt[3 * k + 2] /= w[k];
    }
    it_done = it + 1;
    if (critical) {
      *out_iters = it_done;
      return 2;
    }
    diff = normed_difference(nxt, cur);
    if (out_diffs) out_diffs[it] = diff;
    if (out_pct) {
      // percentage_change: labels of this iteration against the previous one's.
      int64_t changed = 0;
      for (int64_t i = 0; i < ng; i++) changed += map[i] != old_map[i];
      out_pct[it] = 100 * ((double)changed) / ng;
    }
    if (diff < threshold) {
      converged = true;
      break;
    }
    nxt.swap(cur);
    old_map.swap(map);
  }
  // After the loop the reference maps the newest centroids to the grid.  On
  // convergence they are in `nxt`; otherwise the last swap put them in `cur` and the
  // reference swaps them back (src/kmeans.cpp:250-257).  A final diff exactly equal to
  // the threshold takes neither branch and leaves the indices zero-filled.
  std::vector<int> idx(nmu, 0);
  const std::vector<double>* fin = nullptr;
  if (converged) {
    fin = &nxt;
  } else if (diff > threshold) {
    fin = &cur;
  }
  if (fin) {
    classify(fin->data(), nmu, grid, ng, idx.data(), nthreads);
    std::sort(idx.begin(), idx.end());
    std::copy(fin->begin(), fin->end(), out_centroids);
  } else {
    std::copy(cur.begin(), cur.end(), out_centroids);
  }
  std::copy(idx.begin(), idx.end(), out_idx);
  *out_iters = it_done;
  *out_diff = diff;
  if (out_labels) {
    const std::vector<int>& last = converged ? map : old_map;
    std::copy(last.begin(), last.end(), out_labels);
  }
  return 0;
}

int orc_num_threads()
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

}  // extern "C"
