// InterpolatingVectors::IVecs (reference: src/interpolating_vectors.cpp).
//   constructor (:17-57)    reads aoR and fft_grid, truncates the output file when asked,
//                           writes /Hamiltonian/THC/{Orbitals, InterpIndx} as
//                           setup_pseudo_dm does (:75-90)
//                           (complex aoR, k-point orbitals: thc_isdf_complex, Z = |P|^2)
//   kernel (:406-455)       one GPU call (thc_isdf) for the least-squares vectors, the FFT
//                           Coulomb matrix and its Cholesky factor; writes THC/Luv in the
//                           layout of dump_thc_data (:307-315), printing the same warnings
//   dump_qmcpack_data       hcore, Energies, occups, dims, THC/dims (:210-245)
//   rotate = true           the half-rotated variant (:45-49, setup_CZt_half :143-161): reads
//                           aoR_half as well, writes HalfTransformed{Full,Occ}{Orbitals,
//                           InterpIndx}, and kernel writes HalfTransformedMuv (thc_isdf_half;
//                           thc_isdf_half_complex when aoR or aoR_half is complex) instead of
//                           Luv, as dump_thc_data does (:317-328)
// Datasets are written contiguous rather than gzip-chunked (h5helper.cpp:28-35); values and
// shapes are identical.
#include "interpolating_vectors.h"

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <iostream>

#include "../../include/thc_gb300.h"
#include "gpu_context.h"
#include "h5lite.h"

namespace InterpolatingVectors {

IVecs::IVecs(nlohmann::json& input, ContextHandler::BlacsHandler& BH, std::vector<int>& interp_indxs,
             bool rotate, bool append)
{
  (void)BH;
  input_file = input.at("orbital_file").get<std::string>();
  output_file = input.at("output_file").get<std::string>();
  std::cout << "#################################################" << std::endl;
  std::cout << "##   Setting up interpolative vector solver.   ##" << std::endl;
  std::cout << "#################################################" << std::endl;
  std::cout << std::endl;
  half_rotate = rotate;
  prefix = rotate ? "HalfTransformed" : "";
  thc_host::context(&input);
  h5lite::Reader f(input_file);
  // A complex (N_g, n) orbital dataset: its real parts, or (re, im) pairs when an
  // imaginary part is non-zero and complex data are allowed.
  auto read_orbitals = [&](const char* name, std::vector<double>& out, long long& rows,
                           int& cols, bool allow_complex, bool* is_complex) {
    std::vector<uint64_t> dims;
    std::vector<double> aor = f.read_c128(name, &dims);
    rows = (long long)dims[0];
    cols = (int)dims[1];
    double max_im = 0.0;
    for (size_t i = 0; i < (size_t)rows * cols; i++)
      max_im = std::max(max_im, std::fabs(aor[2 * i + 1]));
    if (max_im != 0.0 && allow_complex) {
      *is_complex = true;
      out.swap(aor);
      return;
    }
    if (max_im != 0.0) {
      std::cerr << " * ERROR: " << name << " has a non-zero imaginary part (max " << max_im
                << "); the half-rotated pass takes real orbitals." << std::endl;
      exit(1);
    }
    out.resize((size_t)rows * cols);
    for (size_t i = 0; i < out.size(); i++) out[i] = aor[2 * i];
  };
  read_orbitals("aoR", phi, ngrid, nbasis, true, &complex_orbitals);
  if (complex_orbitals && !rotate)
    std::cout << " * aoR is complex: Z = |P|^2 from complex pseudo-densities." << std::endl;
  if (rotate) {
    long long rows = 0;
    bool occ_complex = false;
    read_orbitals("aoR_half", phi_occ, rows, nocc, true, &occ_complex);
    if (rows != ngrid) {
      std::cerr << " * ERROR: aoR_half has " << rows << " grid points, aoR " << ngrid << std::endl;
      exit(1);
    }
    if (complex_orbitals != occ_complex) {
      // One of the two is real: widen it to (re, 0) pairs for the complex pass.
      std::vector<double>& v = complex_orbitals ? phi_occ : phi;
      std::vector<double> pairs(2 * v.size(), 0.0);
      for (size_t i = 0; i < v.size(); i++) pairs[2 * i] = v[i];
      v.swap(pairs);
      complex_orbitals = true;
    }
    if (complex_orbitals)
      std::cout << " * aoR / aoR_half are complex: Z = P_occ o conj(P) from complex "
                   "pseudo-densities." << std::endl;
  }
  fft_grid = f.read_i32("fft_grid");
  interp = interp_indxs;
  for (int g : interp)
    if (g < 0 || g >= ngrid) {
      std::cerr << " * ERROR: interpolating index " << g << " out of range" << std::endl;
      exit(1);
    }
  h5lite::Writer w(output_file, append);
  // Orbitals at the interpolating points, (n, N_mu, 2), and the indices, under the names
  // setup_pseudo_dm gives them (:75-90).
  int nmu = (int)interp.size();
  auto write_mu = [&](const std::vector<double>& src, int n, const std::string& prfx,
                      bool cplx) {
    std::vector<double> orb((size_t)n * nmu * 2, 0.0);
    for (int i = 0; i < n; i++)
      for (int m = 0; m < nmu; m++) {
        const size_t o = 2 * ((size_t)i * nmu + m);
        if (cplx) {
          orb[o] = src[2 * ((size_t)interp[m] * n + i)];
          orb[o + 1] = src[2 * ((size_t)interp[m] * n + i) + 1];
        } else {
          orb[o] = src[(size_t)interp[m] * n + i];
        }
      }
    std::cout << " * Writing aoR_mu to file" << std::endl;
    w.write_f64("/Hamiltonian/THC/" + prfx + "Orbitals", {(uint64_t)n, (uint64_t)nmu, 2}, orb.data());
    std::cout << " * Writing indices of interpolating points to file" << std::endl;
    w.write_i32("/Hamiltonian/THC/" + prfx + "InterpIndx", {(uint64_t)nmu}, interp.data());
  };
  if (rotate) {
    write_mu(phi, nbasis, prefix + "Full", complex_orbitals);
    write_mu(phi_occ, nocc, prefix + "Occ", complex_orbitals);
  } else {
    write_mu(phi, nbasis, prefix, complex_orbitals);
  }
}

void IVecs::kernel(ContextHandler::BlacsHandler& BH)
{
  (void)BH;
  std::cout << "#################################################" << std::endl;
  std::cout << "##        Finding interpolating vectors.       ##" << std::endl;
  std::cout << "#################################################" << std::endl;
  std::cout << std::endl;
  auto t0 = std::chrono::steady_clock::now();
  h5lite::Reader f(input_file);
  std::vector<double> coul = f.read_f64("fft_coulomb");
  if (fft_grid.size() != 3 || (long long)fft_grid[0] * fft_grid[1] * fft_grid[2] != ngrid)
    std::cout << " * WARNING: FFT grid not consitent with number of real space grid points." << std::endl;
  int nmu = (int)interp.size();
  std::vector<double> L((size_t)nmu * nmu * 2);
  thc_isdf_stats st;
  int status;
  if (half_rotate && complex_orbitals)
    status = thc_isdf_half_complex(thc_host::context(), phi.data(), ngrid, nbasis,
                                   phi_occ.data(), nocc, interp.data(), nmu, fft_grid.data(),
                                   coul.data(), nullptr, nullptr, L.data(), &st);
  else if (half_rotate)
    status = thc_isdf_half(thc_host::context(), phi.data(), ngrid, nbasis, phi_occ.data(), nocc,
                           interp.data(), nmu, fft_grid.data(), coul.data(), -1.0, nullptr,
                           nullptr, L.data(), &st);
  else if (complex_orbitals)
    status = thc_isdf_complex(thc_host::context(), phi.data(), ngrid, nbasis, interp.data(), nmu,
                              fft_grid.data(), coul.data(), -1.0, nullptr, nullptr, L.data(), &st);
  else
    status = thc_isdf(thc_host::context(), phi.data(), ngrid, nbasis, interp.data(), nmu,
                      fft_grid.data(), coul.data(), -1.0, nullptr, nullptr, L.data(), &st);
  if (status != THC_OK && status != THC_ERR_NOT_PD) thc_host::check(status, "ISDF");
  if (st.rank_deficient) {
    std::cout << " * WARNING: CCt matrix is rank deficient (Cholesky pivot " << st.chol_c_info
              << "); regularised with a diagonal shift of " << st.shift_used << std::endl;
    std::cout << std::endl;
  } else {
    std::cout << " * CCt matrix has full rank : " << nmu << std::endl;
    std::cout << std::endl;
  }
  h5lite::Writer w(output_file, false);
  if (half_rotate) {
    // M itself, HalfTransformedMuv (dump_thc_data :317-328).
    std::cout << " * Dumping half transformed Muv data to: " << output_file << "." << std::endl;
    std::cout << std::endl;
    w.write_f64("/Hamiltonian/THC/" + prefix + "Muv", {(uint64_t)nmu, (uint64_t)nmu, 2}, L.data());
    double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    std::cout << " * Time for interpolating vectors and Muv : " << secs << " seconds" << std::endl;
    std::cout << std::endl;
    return;
  }
  std::cout << " * Dumping Luv to: " << output_file << "." << std::endl;
  if (status == THC_ERR_NOT_PD) {
    std::cout << "  * WARNING: Cholesky decomposition failed!" << std::endl;
    std::cout << "  * SCALAPACK Error code: " << st.chol_m_info << std::endl;
    std::cout << "   * The leading minor of order " << st.chol_m_info << " is not positive definite."
              << std::endl;
  }
  w.write_f64("/Hamiltonian/THC/Luv", {(uint64_t)nmu, (uint64_t)nmu, 2}, L.data());
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::cout << " * Time for interpolating vectors and Luv : " << secs << " seconds" << std::endl;
  std::cout << std::endl;
}

void IVecs::dump_qmcpack_data(int thc_cfac, int thc_half_cfac, ContextHandler::BlacsHandler& BH)
{
  (void)BH;
  h5lite::Reader fin(input_file);
  h5lite::Writer w(output_file, false);
  std::vector<uint64_t> dims;
  std::vector<double> hcore = fin.read_c128("hcore", &dims);
  w.write_f64("/Hamiltonian/hcore", {dims[0], dims[1], 2}, hcore.data());
  std::vector<int> num_elec = fin.read_i32("num_electrons");
  int nup = num_elec.at(0), ndown = num_elec.at(1);
  std::vector<double> energy = fin.read_f64("constant_energy_factors");
  w.write_f64("/Hamiltonian/Energies", {1}, energy.data());
  std::vector<int> occups(nup + ndown, 0);
  w.write_i32("/Hamiltonian/occups", {(uint64_t)occups.size()}, occups.data());
  std::vector<int> qmcpack_dims = {-1, 0, 0, nbasis, nup, ndown, 0, 0};
  w.write_i32("/Hamiltonian/dims", {8}, qmcpack_dims.data());
  std::vector<int> thc_dims = {nbasis, thc_cfac * nbasis, thc_half_cfac * nbasis};
  w.write_i32("/Hamiltonian/THC/dims", {3}, thc_dims.data());
}

}  // namespace InterpolatingVectors
