// QRCP::QRCPSolver (reference: src/qrcp.cpp).  The constructor reads the same JSON keys
// (:17-32); kernel() reads aoR (and aoR_half for the half-rotated pass), runs thc_qrcp and
// prints the reference's messages and |R_kk| lines (:100-173).  Differences: the pivots
// come from a pivoted Cholesky factorisation of Z Z^T rather than Householder QR of Z^T
// (the same pivots in exact arithmetic), |R_kk| is printed for the thc_cfac * N_o steps
// taken rather than for all min(rows, N_g).  The indices are 0-based grid indices, as in
// the reference (MatrixOperations::qrcp converts pzgeqpf's 1-based IPIV values with
// add_constant(perm, -1), matrix_operations.h:785-786, before map_perm orders them).
#include "qrcp.h"

#include <chrono>
#include <cmath>
#include <cstdlib>
#include <iomanip>
#include <iostream>

#include "../../include/thc_gb300.h"
#include "gpu_context.h"
#include "h5lite.h"

namespace QRCP {

QRCPSolver::QRCPSolver(nlohmann::json& input, ContextHandler::BlacsHandler& BH)
{
  (void)BH;
  thc_host::context(&input);
  input_file = input.at("orbital_file").get<std::string>();
  try {
    sub_sample = input.at("interpolating_points").at("qrcp").at("sub_sample").get<bool>();
  } catch (nlohmann::json::out_of_range& error) {
    std::cout << " * Performing full QRCP decomposition." << std::endl;
  } catch (nlohmann::json::type_error& error) {
    std::cout << " * Performing full QRCP decomposition." << std::endl;
  }
}

QRCPSolver::~QRCPSolver() {}

namespace {
// A complex (N_g, n) orbital dataset: its real parts, or its (re, im) pairs when an
// imaginary part is non-zero and complex data are allowed (*is_complex set).
std::vector<double> read_orbitals(h5lite::Reader& f, const char* name, long long& rows,
                                  int& cols, bool allow_complex, bool* is_complex)
{
  std::vector<uint64_t> dims;
  std::vector<double> c = f.read_c128(name, &dims);
  rows = (long long)dims[0];
  cols = (int)dims[1];
  double max_im = 0.0;
  for (size_t i = 0; i < (size_t)rows * cols; i++) max_im = std::max(max_im, std::fabs(c[2 * i + 1]));
  if (max_im != 0.0 && allow_complex) {
    *is_complex = true;
    return c;
  }
  if (max_im != 0.0) {
    std::cerr << " * ERROR: " << name << " has a non-zero imaginary part (max " << max_im
              << "); the half-rotated QRCP takes real orbitals." << std::endl;
    exit(1);
  }
  std::vector<double> out((size_t)rows * cols);
  for (size_t i = 0; i < out.size(); i++) out[i] = c[2 * i];
  return out;
}
}  // namespace

void QRCPSolver::kernel(ContextHandler::BlacsHandler& BH, std::vector<int>& interp_indxs,
                        int thc_cfac, bool half_rotate)
{
  (void)BH;
  std::cout << " * Finding interpolating points via QRCP." << std::endl;
  h5lite::Reader f(input_file);
  long long ng = 0, ng_occ = 0;
  int nbasis = 0, nelec = 0;
  bool cplx = false, unused = false;
  std::vector<double> phi = read_orbitals(f, "aoR", ng, nbasis, !half_rotate, &cplx);
  std::vector<double> occ;
  std::cout << " * Constructing Z matrix." << std::endl;
  if (half_rotate) {
    occ = read_orbitals(f, "aoR_half", ng_occ, nelec, false, &unused);
    if (ng_occ != ng) {
      std::cerr << " * ERROR: aoR_half has " << ng_occ << " grid points, aoR " << ng << std::endl;
      exit(1);
    }
  }
  const int num_interp_pts = thc_cfac * nbasis;
  if (num_interp_pts <= 0 || num_interp_pts > ng) {
    std::cerr << " * ERROR: thc_cfac * nbasis = " << num_interp_pts << " points for " << ng
              << " grid points" << std::endl;
    exit(1);
  }
  auto t0 = std::chrono::steady_clock::now();
  interp_indxs.resize(num_interp_pts);
  std::vector<double> diag(num_interp_pts);
  thc_qrcp_stats st;
  int status = cplx ? thc_qrcp_complex(thc_host::context(), phi.data(), ng, nbasis,
                                        num_interp_pts, interp_indxs.data(), nullptr,
                                        diag.data(), &st)
                    : thc_qrcp(thc_host::context(), phi.data(), ng, nbasis,
                               half_rotate ? occ.data() : nullptr, nelec, num_interp_pts,
                               interp_indxs.data(), nullptr, diag.data(), &st);
  thc_host::check(status, "QRCP");
  double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::cout << "  * Time for QRCP: " << secs << " seconds (numerical rank " << st.numerical_rank
            << ")." << std::endl;
  const std::string prefix = half_rotate ? "half_ix" : "full_ix";
  for (int i = 0; i < num_interp_pts; i++)
    std::cout << prefix + "_diag" << " " << i << " " << std::setprecision(16) << diag[i] << std::endl;
}

}  // namespace QRCP
