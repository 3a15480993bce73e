// KMeans::KMeansSolver (reference: src/kmeans.cpp).  The constructor reads the same JSON
// keys with the same defaults (:16-44); kernel() reads the grid, density and aoR shape from
// the orbital file (:190-197), draws the initial points with std::shuffle(mt19937) on the
// host and runs the iteration on the GPU (thc_kmeans), printing the reference's progress
// table (:232-238) from the device's iteration history.
#include "kmeans.h"

#include <chrono>
#include <cstdlib>
#include <iomanip>
#include <iostream>

#include "../../include/thc_gb300.h"
#include "gpu_context.h"
#include "h5lite.h"

namespace KMeans {

KMeansSolver::KMeansSolver(nlohmann::json& input, ContextHandler::BlacsHandler& BH)
{
  (void)BH;
  filename = input.at("orbital_file").get<std::string>();
  nlohmann::json kmeans = input.at("interpolating_points").at("kmeans");
  max_it = kmeans.at("max_it").get<int>();
  threshold = kmeans.at("threshold").get<double>();
  try {
    rng_seed = (unsigned int)kmeans.at("rng_seed").get<int>();
  } catch (nlohmann::json::out_of_range& error) {
    std::cout << " * RNG seed not set in input file." << std::endl;
    rng_seed = (unsigned int)std::chrono::system_clock::now().time_since_epoch().count();
    std::cout << " * Setting RNG seed to : " << rng_seed << std::endl;
    std::cout << std::endl;
  }
  try {
    density_label = kmeans.at("density").get<std::string>();
  } catch (nlohmann::json::out_of_range& error) {
    density_label = "density";
    std::cout << " * Density not specified." << std::endl;
    std::cout << " * Using full basis set for density." << std::endl;
  }
  thc_host::context(&input);
}

KMeansSolver::~KMeansSolver() {}

void KMeansSolver::kernel(ContextHandler::BlacsHandler& BH, std::vector<int>& interp_indxs,
                          int thc_cfac)
{
  (void)BH;
  auto t0 = std::chrono::steady_clock::now();
  h5lite::Reader f(filename);
  std::vector<uint64_t> gdims, ddims;
  std::vector<double> grid = f.read_f64("real_space_grid", &gdims);
  std::vector<double> rho = f.read_f64(density_label, &ddims);
  std::vector<uint64_t> adims = f.info("aoR").dims;
  int num_interp_pts = thc_cfac * (int)adims[1];
  long long num_grid_pts = (long long)adims[0];
  if ((long long)gdims[0] != num_grid_pts || gdims.size() != 2 || gdims[1] != 3 ||
      (long long)rho.size() != num_grid_pts) {
    std::cerr << " * ERROR: real_space_grid / " << density_label << " / aoR shapes disagree" << std::endl;
    exit(1);
  }
  interp_indxs.resize(num_interp_pts);
  std::cout << "#################################################" << std::endl;
  std::cout << "## Finding interpolation points using K-Means. ##" << std::endl;
  std::cout << "#################################################" << std::endl;
  std::cout << std::endl;
  std::cout << " * Number of interpolating points : " << num_interp_pts << std::endl;
  std::cout << " * Number of grid points : " << num_grid_pts << std::endl;
  std::vector<int> init(num_interp_pts);
  thc_host::check(thc_kmeans_initial_indices(num_grid_pts, num_interp_pts, rng_seed, init.data()),
                  "initial centroids");
  thc_ctx* ctx = thc_host::context();
  thc_kmeans_stats st;
  int status = thc_kmeans(ctx, grid.data(), rho.data(), num_grid_pts, num_interp_pts, init.data(),
                          max_it, threshold, interp_indxs.data(), &st);
  if (status == THC_ERR_EMPTY_CLUSTER) {
    // Reference behaviour (src/kmeans.cpp:137-143).
    std::cout << " CRITICAL ERROR: Found centroid with weight ~ 0" << std::endl;
    exit(1);
  }
  thc_host::check(status, "k-means");
  std::vector<double> diff(st.iterations), pct(st.iterations);
  if (st.iterations > 0 &&
      thc_kmeans_history(ctx, diff.data(), pct.data(), st.iterations) == THC_OK) {
    std::cout << "  *   Step        Error     % change" << std::endl;
    for (int i = 0; i < st.iterations; i++)
      if (i % 10 == 0)
        std::cout << std::setw(10) << i << "  " << std::setprecision(5) << std::scientific
                  << diff[i] << "  " << pct[i] << std::endl;
    std::cout.unsetf(std::ios::floatfield);
  }
  if (!st.converged)
    std::cout << " * Threshold not breached. Final Error: " << st.final_diff << std::endl;
  if (st.duplicates) std::cout << "ERROR: Found repeated indices: " << st.duplicates << std::endl;
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::cout << " * Time taken for K-Means solution: " << secs << " seconds" << std::endl;
  std::cout << std::endl;
}

}  // namespace KMeans
