// extern "C" entry points over the reference's own L0 math files
// (src/flare_pp/radial.cpp, cutoffs.cpp, y_grad.cpp, descriptors/wigner3j.cpp),
// compiled unmodified
// from the reference tree by oracle/ref/build_ref.sh.  Used only to record
// golden vectors that pin the oracle's restatement.
#include <cstring>
#include <string>
#include <vector>
#include <complex>
#include "radial.h"
#include "cutoffs.h"
#include "y_grad.h"
#include "wigner3j.h"

extern "C" {

// get_Y (y_grad.cpp:667): real harmonics and gradients, (l+1)^2 each.
void ref_get_Y(double x, double y, double z, int lmax, double *Y, double *Yx,
               double *Yy, double *Yz) {
  int H = (lmax + 1) * (lmax + 1);
  std::vector<double> a(H, 0), b(H, 0), c(H, 0), d(H, 0);
  get_Y(a, b, c, d, x, y, z, lmax);
  std::memcpy(Y, a.data(), H * sizeof(double));
  std::memcpy(Yx, b.data(), H * sizeof(double));
  std::memcpy(Yy, c.data(), H * sizeof(double));
  std::memcpy(Yz, d.data(), H * sizeof(double));
}

// get_complex_Y (y_grad.cpp:24): complex harmonics, interleaved re/im.
void ref_get_complex_Y(double x, double y, double z, int lmax, double *Y,
                       double *Yx, double *Yy, double *Yz) {
  Eigen::VectorXcd a, b, c, d;
  get_complex_Y(a, b, c, d, x, y, z, lmax);
  int H = (lmax + 1) * (lmax + 1);
  for (int i = 0; i < H; i++) {
    Y[2 * i] = a(i).real(); Y[2 * i + 1] = a(i).imag();
    Yx[2 * i] = b(i).real(); Yx[2 * i + 1] = b(i).imag();
    Yy[2 * i] = c(i).real(); Yy[2 * i + 1] = c(i).imag();
    Yz[2 * i] = d(i).real(); Yz[2 * i + 1] = d(i).imag();
  }
}

// calculate_radial (radial.cpp:344) with a named basis and cutoff function.
int ref_calculate_radial(const char *basis, const char *cutoff, double x,
                         double y, double z, double r, double rcut, int N,
                         double r1, double *g, double *gx, double *gy,
                         double *gz) {
  std::function<void(std::vector<double> &, std::vector<double> &, double, int,
                     std::vector<double>)> bf;
  std::function<void(std::vector<double> &, double, double,
                     std::vector<double>)> cf;
  set_radial_basis(std::string(basis), bf);
  set_cutoff(std::string(cutoff), cf);
  if (!bf || !cf) return -1;
  std::vector<double> a(N, 0), b(N, 0), c(N, 0), d(N, 0);
  std::vector<double> radial_hyps{r1, rcut};
  std::vector<double> cutoff_hyps;
  calculate_radial(a, b, c, d, bf, cf, x, y, z, r, rcut, N, radial_hyps,
                   cutoff_hyps);
  std::memcpy(g, a.data(), N * sizeof(double));
  std::memcpy(gx, b.data(), N * sizeof(double));
  std::memcpy(gy, c.data(), N * sizeof(double));
  std::memcpy(gz, d.data(), N * sizeof(double));
  return 0;
}

// compute_coeffs (wigner3j.cpp:5): the (lmax+1)^6 table of Wigner 3j symbols.
int ref_compute_coeffs(int lmax, double *out, long n) {
  Eigen::VectorXd w = compute_coeffs(lmax);
  if (w.size() != n) return -1;
  for (long i = 0; i < n; i++) out[i] = w(i);
  return 0;
}
}
