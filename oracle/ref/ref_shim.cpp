// extern "C" entry points over the reference's own L0 math files
// (src/flare_pp/radial.cpp, cutoffs.cpp, y_grad.cpp, descriptors/wigner3j.cpp)
// and its per-atom pair-style math (lammps_plugins/lammps_descriptor.cpp),
// compiled unmodified from the reference tree by oracle/ref/build_ref.sh.
// Used only to record golden vectors that pin the oracle's restatement.
#include <cstring>
#include <string>
#include <vector>
#include <complex>
#include "radial.h"
#include "cutoffs.h"
#include "y_grad.h"
#include "wigner3j.h"
#include "lammps_descriptor.h"

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

// The per-atom loop of PairFLARE::compute (lammps_plugins/pair_flare.cpp:
// 95-180) over LAMMPS-shaped arrays, driving the reference's own
// single_bond_multiple_cutoffs, B2_descriptor and compute_energy_and_u
// (lammps_descriptor.cpp:7-304).  The loop itself (count of pairs inside
// the cutoff, skip of empty environments below 1e-8, f_ij = dA/dr_ij . u
// added to f_i and taken from f_j, the virial of ev_tally_xyz with newton_pair
// on, the per-atom energy of ev_tally_full) is restated here because
// pair_flare.cpp needs LAMMPS to compile.
//   x nall x 3, type nall (1-based), neighbors of atom i at
//   neighbors[nbr_offset[i] .. nbr_offset[i] + numneigh[i]) (atom indices),
//   cutoffs n_species x n_species (row-major), beta per species n_d x n_d
//   (power 2, dense symmetric) or n_d (power 1).
//   Outputs: f nall x 3 (added to), eatom nall (added to), virial[6]
//   (xx, yy, zz, xy, xz, yz; added to).  For the first n_rec listed atoms
//   the single-bond values, B2 values, u and E_i go to rec_* (rows of
//   n_bond, n_d, n_bond, 1).
int ref_pair_flare(int nall, const double *x, const int *type, int inum, const int *ilist,
                   const int *numneigh, const int *nbr_offset, const int *neighbors,
                   int n_species, int N, int lmax, double r1, const double *cutoffs,
                   const char *cutoff_name, int power, const double *beta, double *f,
                   double *eatom, double *virial, int n_rec, double *rec_sb, double *rec_b2,
                   double *rec_u, double *rec_e) {
  std::function<void(std::vector<double> &, std::vector<double> &, double, int,
                     std::vector<double>)> basis;
  std::function<void(std::vector<double> &, double, double, std::vector<double>)> cutf;
  set_radial_basis(std::string("chebyshev"), basis);
  set_cutoff(std::string(cutoff_name), cutf);
  if (!basis || !cutf || (power != 1 && power != 2)) return -1;
  const int n_rad = n_species * N, H = (lmax + 1) * (lmax + 1);
  const int n_bond = n_rad * H, n_d = n_rad * (n_rad + 1) / 2 * (lmax + 1);
  std::vector<double *> xp(nall);
  for (int k = 0; k < nall; k++) xp[k] = const_cast<double *>(x + 3 * k);
  std::vector<int> tp(type, type + nall);
  std::vector<int> nb(neighbors, neighbors + (inum > 0 ? nbr_offset[inum] : 0));
  Eigen::MatrixXd cut(n_species, n_species);
  double rc_max = 0;
  for (int a = 0; a < n_species; a++)
    for (int b = 0; b < n_species; b++) {
      cut(a, b) = cutoffs[a * n_species + b];
      if (cut(a, b) > rc_max) rc_max = cut(a, b);
    }
  const int bcols = power == 1 ? 1 : n_d;
  std::vector<Eigen::MatrixXd> betas;
  for (int s = 0; s < n_species; s++) {
    Eigen::MatrixXd B(n_d, bcols);
    for (int r = 0; r < n_d; r++)
      for (int c = 0; c < bcols; c++) B(r, c) = beta[(size_t)s * n_d * bcols + (size_t)r * bcols + c];
    betas.push_back(B);
  }
  std::vector<double> radial_hyps{r1, rc_max}, cutoff_hyps;
  Eigen::VectorXd sbv, b2v, u;
  Eigen::MatrixXd sbd;
  for (int ii = 0; ii < inum; ii++) {
    const int i = ilist[ii];
    const int jnum = numneigh[i];
    int *jlist = nb.data() + nbr_offset[i];
    const double xt = x[3 * i], yt = x[3 * i + 1], zt = x[3 * i + 2];
    const int ti = type[i] - 1;
    int n_inner = 0;
    for (int jj = 0; jj < jnum; jj++) {
      const int j = jlist[jj];
      const double rc = cut(ti, type[j] - 1);
      const double dx = x[3 * j] - xt, dy = x[3 * j + 1] - yt, dz = x[3 * j + 2] - zt;
      if (dx * dx + dy * dy + dz * dz < rc * rc) n_inner++;
    }
    single_bond_multiple_cutoffs(xp.data(), tp.data(), jnum, n_inner, i, xt, yt, zt, jlist,
                                 basis, cutf, n_species, N, lmax, radial_hyps, cutoff_hyps,
                                 sbv, sbd, cut);
    double nsq = 0, evdwl = 0;
    B2_descriptor(b2v, nsq, sbv, n_species, N, lmax);
    compute_energy_and_u(b2v, nsq, sbv, power, n_species, N, lmax, betas[ti], u, &evdwl);
    if (ii < n_rec) {
      for (int k = 0; k < n_bond; k++) rec_sb[(size_t)ii * n_bond + k] = sbv(k);
      for (int k = 0; k < n_d; k++) rec_b2[(size_t)ii * n_d + k] = b2v(k);
      for (int k = 0; k < n_bond; k++) rec_u[(size_t)ii * n_bond + k] = u(k);
      rec_e[ii] = nsq < 1e-8 ? 0.0 : evdwl;
    }
    if (nsq < 1e-8) continue;
    int n_count = 0;
    for (int jj = 0; jj < jnum; jj++) {
      const int j = jlist[jj];
      const double rc = cut(ti, type[j] - 1);
      const double dx = xt - x[3 * j], dy = yt - x[3 * j + 1], dz = zt - x[3 * j + 2];
      if (dx * dx + dy * dy + dz * dz < rc * rc) {
        double fr[3];
        for (int a = 0; a < 3; a++) {
          double acc = 0;
          for (int k = 0; k < n_bond; k++) acc += sbd(3 * n_count + a, k) * u(k);
          fr[a] = acc;
        }
        for (int a = 0; a < 3; a++) {
          f[3 * i + a] += fr[a];
          f[3 * j + a] -= fr[a];
        }
        virial[0] += dx * fr[0];
        virial[1] += dy * fr[1];
        virial[2] += dz * fr[2];
        virial[3] += dx * fr[1];
        virial[4] += dx * fr[2];
        virial[5] += dy * fr[2];
        n_count++;
      }
    }
    eatom[i] += evdwl;
  }
  return 0;
}
}
