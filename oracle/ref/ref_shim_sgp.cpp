// extern "C" entry points over the reference's SparseGP (bffs/sparse_gp.cpp)
// with NormalizedDotProduct kernels, compiled unmodified from the reference
// tree by oracle/ref/build_ref.sh against the Eigen and nlohmann_json
// stand-ins in oracle/ref/stub.  Used only to record golden vectors that pin
// the oracle's sparse GP restatement (training labels and their order, Kuu,
// Kuf, the QR solve, the likelihood and its gradient, hyperparameter updates,
// predictions and cluster uncertainties).
//
// Structures here carry any number of descriptors (handles of ref_b2_new /
// ref_b3_new) and their labels; handles are owned by the caller (ref_*_free).
// Matrices are returned row-major; a getter called with a null output
// returns the element count (negative for an unknown field).
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "descriptor.h"
#include "normalized_dot_product.h"
#include "sparse_gp.h"
#include "structure.h"

namespace {

struct RefSGP {
  std::vector<NormalizedDotProduct *> kernels;
  SparseGP *gp = nullptr;
};

template <typename M> int put_rows(const M &m, double *out, int *rows, int *cols) {
  if (rows) *rows = (int)m.rows();
  if (cols) *cols = (int)m.cols();
  if (out)
    for (long i = 0; i < m.rows(); i++)
      for (long j = 0; j < m.cols(); j++) out[i * m.cols() + j] = m(i, j);
  return (int)(m.rows() * m.cols());
}

Eigen::VectorXd vec(const double *v, int n) {
  Eigen::VectorXd x(n);
  for (int i = 0; i < n; i++) x(i) = v[i];
  return x;
}

}  // namespace

extern "C" {

// Structure(cell, species, positions, cutoff, descriptors) (structure.h:92-97)
void *ref_sgp_structure_new(const double *cell, const int *species, const double *pos, int noa,
                            double cutoff, void **descs, int n_desc) {
  Eigen::MatrixXd c(3, 3), p(noa, 3);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c(i, j) = cell[3 * i + j];
  for (int i = 0; i < noa; i++)
    for (int j = 0; j < 3; j++) p(i, j) = pos[3 * i + j];
  std::vector<int> sp(species, species + noa);
  std::vector<Descriptor *> calc;
  for (int k = 0; k < n_desc; k++) calc.push_back(static_cast<Descriptor *>(descs[k]));
  return new Structure(c, sp, p, cutoff, calc);
}

void ref_sgp_structure_free(void *s) { delete static_cast<Structure *>(s); }

// energy (ne), forces (nf), stresses (ns) labels (structure.h:67)
void ref_sgp_structure_set_labels(void *s, const double *e, int ne, const double *f, int nf,
                                  const double *st, int ns) {
  Structure &x = *static_cast<Structure *>(s);
  x.energy = vec(e, ne);
  x.forces = vec(f, nf);
  x.stresses = vec(st, ns);
}

// mean_efs / variance_efs of a structure after a prediction
int ref_sgp_structure_get(void *s, const char *field, double *out) {
  const Structure &x = *static_cast<Structure *>(s);
  const std::string f(field);
  if (f == "mean_efs") return put_rows(x.mean_efs, out, nullptr, nullptr);
  if (f == "variance_efs") return put_rows(x.variance_efs, out, nullptr, nullptr);
  return -1;
}

// SparseGP({NormalizedDotProduct(sigma_k, power_k)}, energy, force, stress noise)
void *ref_sgp_new(int n_kernels, const double *sigmas, const double *powers, double e_noise,
                  double f_noise, double s_noise) {
  auto *h = new RefSGP;
  std::vector<Kernel *> ks;
  for (int k = 0; k < n_kernels; k++) {
    h->kernels.push_back(new NormalizedDotProduct(sigmas[k], powers[k]));
    ks.push_back(h->kernels.back());
  }
  h->gp = new SparseGP(ks, e_noise, f_noise, s_noise);
  return h;
}

void ref_sgp_free(void *h) {
  auto *r = static_cast<RefSGP *>(h);
  delete r->gp;
  for (auto *k : r->kernels) delete k;
  delete r;
}

// add_training_structure(structure, atom_indices) (n_atoms < 0: {-1}, all atoms)
void ref_sgp_add_training_structure(void *h, void *s, const int *atoms, int n_atoms) {
  std::vector<int> a = n_atoms < 0 ? std::vector<int>{-1} : std::vector<int>(atoms, atoms + n_atoms);
  static_cast<RefSGP *>(h)->gp->add_training_structure(*static_cast<Structure *>(s), a);
}

void ref_sgp_add_specific_environments(void *h, void *s, const int *atoms, int n) {
  static_cast<RefSGP *>(h)->gp->add_specific_environments(*static_cast<Structure *>(s),
                                                          std::vector<int>(atoms, atoms + n));
}

void ref_sgp_update_matrices_QR(void *h) { static_cast<RefSGP *>(h)->gp->update_matrices_QR(); }

void ref_sgp_set_hyperparameters(void *h, const double *hyps, int n) {
  static_cast<RefSGP *>(h)->gp->set_hyperparameters(vec(hyps, n));
}

void ref_sgp_compute_likelihood_stable(void *h) {
  static_cast<RefSGP *>(h)->gp->compute_likelihood_stable();
}

double ref_sgp_compute_likelihood_gradient_stable(void *h) {
  return static_cast<RefSGP *>(h)->gp->compute_likelihood_gradient_stable(false);
}

// what = "mean", "SOR", "DTC"
int ref_sgp_predict(void *h, const char *what, void *s) {
  SparseGP &gp = *static_cast<RefSGP *>(h)->gp;
  Structure &x = *static_cast<Structure *>(s);
  const std::string w(what);
  if (w == "mean") gp.predict_mean(x);
  else if (w == "SOR") gp.predict_SOR(x);
  else if (w == "DTC") gp.predict_DTC(x);
  else return -1;
  return 0;
}

// compute_cluster_uncertainties(structure)[kernel] (sparse_gp.cpp:93-133)
int ref_sgp_cluster_uncertainties(void *h, void *s, int kernel, double *out) {
  SparseGP &gp = *static_cast<RefSGP *>(h)->gp;
  std::vector<Eigen::VectorXd> v = gp.compute_cluster_uncertainties(*static_cast<Structure *>(s));
  if (kernel < 0 || kernel >= (int)v.size()) return -1;
  return put_rows(v[kernel], out, nullptr, nullptr);
}

// NormalizedDotProduct::compute_mapping_coefficients (power 1 or 2) and
// compute_varmap_coefficients (power 1) of kernel k of the trained GP
// (normalized_dot_product.cpp:624-850).
int ref_sgp_mapping_coefficients(void *h, int k, double *out, int *rows, int *cols) {
  RefSGP &r = *static_cast<RefSGP *>(h);
  if (k < 0 || k >= (int)r.kernels.size()) return -1;
  return put_rows(r.kernels[k]->compute_mapping_coefficients(*r.gp, k), out, rows, cols);
}

int ref_sgp_varmap_coefficients(void *h, int k, double *out, int *rows, int *cols) {
  RefSGP &r = *static_cast<RefSGP *>(h);
  if (k < 0 || k >= (int)r.kernels.size()) return -1;
  return put_rows(r.kernels[k]->compute_varmap_coefficients(*r.gp, k), out, rows, cols);
}

// Matrices and vectors of the GP: "Kuu", "Kuf", "alpha", "R_inv", "L_inv",
// "y", "noise_vector", "hyperparameters", "likelihood_gradient"; scalars
// "log_marginal_likelihood", "data_fit", "complexity_penalty".
int ref_sgp_get(void *h, const char *field, double *out, int *rows, int *cols) {
  const SparseGP &gp = *static_cast<RefSGP *>(h)->gp;
  const std::string f(field);
  if (f == "Kuu") return put_rows(gp.Kuu, out, rows, cols);
  if (f == "Kuf") return put_rows(gp.Kuf, out, rows, cols);
  if (f == "alpha") return put_rows(gp.alpha, out, rows, cols);
  if (f == "R_inv") return put_rows(gp.R_inv, out, rows, cols);
  if (f == "L_inv") return put_rows(gp.L_inv, out, rows, cols);
  if (f == "y") return put_rows(gp.y, out, rows, cols);
  if (f == "noise_vector") return put_rows(gp.noise_vector, out, rows, cols);
  if (f == "hyperparameters") return put_rows(gp.hyperparameters, out, rows, cols);
  if (f == "likelihood_gradient") return put_rows(gp.likelihood_gradient, out, rows, cols);
  double v;
  if (f == "log_marginal_likelihood") v = gp.log_marginal_likelihood;
  else if (f == "data_fit") v = gp.data_fit;
  else if (f == "complexity_penalty") v = gp.complexity_penalty;
  else return -1;
  if (rows) *rows = 1;
  if (cols) *cols = 1;
  if (out) out[0] = v;
  return 1;
}
}
