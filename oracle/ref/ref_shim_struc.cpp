// extern "C" entry points over the reference's Structure (structure.cpp),
// B2 and B3 (descriptors/b2.cpp, descriptors/b3.cpp, descriptors/descriptor.cpp) and
// NormalizedDotProduct (kernels/normalized_dot_product.cpp), compiled
// unmodified from the reference tree by oracle/ref/build_ref.sh against the
// Eigen and nlohmann_json stand-ins in oracle/ref/stub.  Used only to record
// golden vectors that pin the oracle's neighbor list, DescriptorValues and
// kernel restatements.
//
// Handles are opaque pointers owned by the caller (ref_*_free).  Matrices are
// returned row-major; a getter called with a null output returns the element
// count, otherwise it fills the output and returns the count (negative on an
// unknown field or index).
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "b2.h"
#include "b3.h"
#include "descriptor.h"
#include "normalized_dot_product.h"
#include "structure.h"

namespace {

template <typename M> int copy_rows(const M &m, double *out) {
  const int n = (int)(m.rows() * m.cols());
  if (out)
    for (long i = 0; i < m.rows(); i++)
      for (long j = 0; j < m.cols(); j++) out[i * m.cols() + j] = m(i, j);
  return n;
}

template <typename V> int copy_int(const V &v, int *out) {
  const int n = (int)v.size();
  if (out)
    for (int i = 0; i < n; i++) out[i] = v(i);
  return n;
}

struct RefStructure {
  Structure *s = nullptr;
};

}  // namespace

extern "C" {

// Descriptor handles are Descriptor pointers (ref_structure_new takes either).
// B2(radial_basis = "chebyshev", cutoff_function, radial_hyps = {r1, rc},
//    cutoff_hyps = {}, descriptor_settings = {ns, N, lmax}, cutoffs) (b2.h:34-46).
void *ref_b2_new(int ns, int N, int lmax, double r1, double rc, const double *cutoffs,
                 const char *cutoff_name) {
  Eigen::MatrixXd cut(ns, ns);
  for (int a = 0; a < ns; a++)
    for (int b = 0; b < ns; b++) cut(a, b) = cutoffs[a * ns + b];
  Descriptor *d = new B2("chebyshev", cutoff_name, std::vector<double>{r1, rc},
                         std::vector<double>{}, std::vector<int>{ns, N, lmax}, cut);
  return d;
}

void ref_b2_free(void *b2) { delete static_cast<B2 *>(static_cast<Descriptor *>(b2)); }

// B3(radial_basis = "chebyshev", cutoff_function, radial_hyps = {r1, rc},
//    cutoff_hyps = {}, descriptor_settings = {ns, N, lmax}) (b3.h:27-30).
void *ref_b3_new(int ns, int N, int lmax, double r1, double rc, const char *cutoff_name) {
  Descriptor *d = new B3("chebyshev", cutoff_name, std::vector<double>{r1, rc},
                         std::vector<double>{}, std::vector<int>{ns, N, lmax});
  return d;
}

void ref_b3_free(void *b3) { delete static_cast<B3 *>(static_cast<Descriptor *>(b3)); }

// Structure(cell, species, positions, cutoff, {descriptor}) (structure.h:92-97):
// neighbors (structure.cpp:52-118) and, with a descriptor (a handle of
// ref_b2_new or ref_b3_new), its values.
// cell: 3 x 3 row-major, rows are the lattice vectors; positions noa x 3.
void *ref_structure_new(const double *cell, const int *species, const double *pos, int noa,
                        double cutoff, void *desc) {
  Eigen::MatrixXd c(3, 3), p(noa, 3);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) c(i, j) = cell[3 * i + j];
  for (int i = 0; i < noa; i++)
    for (int j = 0; j < 3; j++) p(i, j) = pos[3 * i + j];
  std::vector<int> sp(species, species + noa);
  std::vector<Descriptor *> calc;
  if (desc) calc.push_back(static_cast<Descriptor *>(desc));
  auto *r = new RefStructure;
  r->s = new Structure(c, sp, p, cutoff, calc);
  return r;
}

void ref_structure_free(void *h) {
  auto *r = static_cast<RefStructure *>(h);
  delete r->s;
  delete r;
}

// Structure fields: "relative_positions" (n x 4), "wrapped_positions"
// (noa x 3), "volume", "single_sweep_cutoff", "sweep".
int ref_structure_dbl(void *h, const char *field, double *out) {
  const Structure &s = *static_cast<RefStructure *>(h)->s;
  const std::string f(field);
  if (f == "relative_positions") return copy_rows(s.relative_positions, out);
  if (f == "wrapped_positions") return copy_rows(s.wrapped_positions, out);
  double v;
  if (f == "volume") v = s.volume;
  else if (f == "single_sweep_cutoff") v = s.single_sweep_cutoff;
  else if (f == "sweep") v = s.sweep;
  else return -1;
  if (out) out[0] = v;
  return 1;
}

// "neighbor_count", "cumulative_neighbor_count", "structure_indices",
// "neighbor_species".
int ref_structure_int(void *h, const char *field, int *out) {
  const Structure &s = *static_cast<RefStructure *>(h)->s;
  const std::string f(field);
  if (f == "neighbor_count") return copy_int(s.neighbor_count, out);
  if (f == "cumulative_neighbor_count") return copy_int(s.cumulative_neighbor_count, out);
  if (f == "structure_indices") return copy_int(s.structure_indices, out);
  if (f == "neighbor_species") return copy_int(s.neighbor_species, out);
  return -1;
}

// DescriptorValues (descriptor.h:31-57) of the structure's descriptor, per
// species: "descriptors", "descriptor_force_dervs", "neighbor_coordinates"
// (matrices), "descriptor_norms", "descriptor_force_dots", "cutoff_values"
// (vectors); "n_cols" gives the column count of a matrix field.
int ref_dv_dbl(void *h, const char *field, int s, double *out) {
  const Structure &st = *static_cast<RefStructure *>(h)->s;
  if (st.descriptors.empty()) return -2;
  const DescriptorValues &d = st.descriptors[0];
  if (s < 0 || s >= d.n_types) return -3;
  const std::string f(field);
  if (f == "descriptors") return copy_rows(d.descriptors[s], out);
  if (f == "descriptor_force_dervs") return copy_rows(d.descriptor_force_dervs[s], out);
  if (f == "neighbor_coordinates") return copy_rows(d.neighbor_coordinates[s], out);
  if (f == "descriptor_norms") return copy_rows(d.descriptor_norms[s], out);
  if (f == "descriptor_force_dots") return copy_rows(d.descriptor_force_dots[s], out);
  if (f == "cutoff_values") return copy_rows(d.cutoff_values[s], out);
  if (f == "volume") {
    if (out) out[0] = d.volume;
    return 1;
  }
  return -1;
}

// "neighbor_counts", "cumulative_neighbor_counts", "atom_indices",
// "neighbor_indices" per species; "n_descriptors", "n_types", "n_atoms"
// (s ignored).
int ref_dv_int(void *h, const char *field, int s, int *out) {
  const Structure &st = *static_cast<RefStructure *>(h)->s;
  if (st.descriptors.empty()) return -2;
  const DescriptorValues &d = st.descriptors[0];
  const std::string f(field);
  int v;
  if (f == "n_descriptors") v = d.n_descriptors;
  else if (f == "n_types") v = d.n_types;
  else if (f == "n_atoms") v = d.n_atoms;
  else {
    if (s < 0 || s >= d.n_types) return -3;
    if (f == "neighbor_counts") return copy_int(d.neighbor_counts[s], out);
    if (f == "cumulative_neighbor_counts") return copy_int(d.cumulative_neighbor_counts[s], out);
    if (f == "atom_indices") return copy_int(d.atom_indices[s], out);
    if (f == "neighbor_indices") return copy_int(d.neighbor_indices[s], out);
    return -1;
  }
  if (out) out[0] = v;
  return 1;
}

// ClusterDescriptor (descriptor.h:61-90): an empty set of n_types x n_d,
// then add_clusters_by_type from a structure's DescriptorValues with the
// atoms of each type given per type (indices within the type).
void *ref_cluster_new(int n_types, int n_d) {
  auto *c = new ClusterDescriptor();
  c->initialize_cluster(n_types, n_d);
  return c;
}

void ref_cluster_free(void *c) { delete static_cast<ClusterDescriptor *>(c); }

int ref_cluster_add(void *c, void *h, const int *counts, const int *flat) {
  const Structure &st = *static_cast<RefStructure *>(h)->s;
  if (st.descriptors.empty()) return -2;
  const DescriptorValues &d = st.descriptors[0];
  std::vector<std::vector<int>> cl(d.n_types);
  int k = 0;
  for (int s = 0; s < d.n_types; s++)
    for (int q = 0; q < counts[s]; q++) cl[s].push_back(flat[k++]);
  static_cast<ClusterDescriptor *>(c)->add_clusters_by_type(d, cl);
  return 0;
}

// NormalizedDotProduct(sigma, power) (normalized_dot_product.h:18) kernels:
//   what = "envs_envs" (a, b clusters), "envs_struc" (a cluster, b structure),
//   "struc_struc" (a, b structures), "self_kernel_struc" (a structure).
// Returns the element count (-2 where the reference throws); with rows
// non-null stores the shape.
int ref_kernel(const char *what, double sigma, double power, void *a, void *b, double *out,
               int *rows, int *cols) {
  NormalizedDotProduct k(sigma, power);
  const std::string w(what);
  Eigen::MatrixXd m;
  try {
  if (w == "envs_envs") {
    m = k.envs_envs(*static_cast<ClusterDescriptor *>(a), *static_cast<ClusterDescriptor *>(b),
                    k.kernel_hyperparameters);
  } else if (w == "envs_struc") {
    m = k.envs_struc(*static_cast<ClusterDescriptor *>(a),
                     static_cast<RefStructure *>(b)->s->descriptors[0], k.kernel_hyperparameters);
  } else if (w == "struc_struc") {
    m = k.struc_struc(static_cast<RefStructure *>(a)->s->descriptors[0],
                      static_cast<RefStructure *>(b)->s->descriptors[0],
                      k.kernel_hyperparameters);
  } else if (w == "self_kernel_struc") {
    m = k.self_kernel_struc(static_cast<RefStructure *>(a)->s->descriptors[0],
                            k.kernel_hyperparameters);
  } else {
    return -1;
  }
  } catch (const std::exception &) {
    // the reference throws (struc_struc with power < 2 and a zero dot product)
    return -2;
  }
  if (rows) {
    *rows = (int)m.rows();
    *cols = (int)m.cols();
  }
  return copy_rows(m, out);
}
}
