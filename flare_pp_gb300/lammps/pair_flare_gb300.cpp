// PairFLAREGB300: see pair_flare_gb300.h.
#include "pair_flare_gb300.h"

#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace {

void check(int rc, const char *what) {
  if (rc != FPP_OK)
    throw std::runtime_error(std::string(what) + ": " + fpp_last_error());
}

// Whole lines until n numbers have been read (PairFLARE::grab).
std::vector<double> grab(std::istream &in, size_t n) {
  std::vector<double> out;
  std::string line;
  while (out.size() < n && std::getline(in, line)) {
    std::istringstream ls(line);
    double v;
    while (ls >> v) out.push_back(v);
  }
  if (out.size() < n) throw std::runtime_error("potential file ends early");
  out.resize(n);
  return out;
}

}  // namespace

PairFLAREGB300::PairFLAREGB300(int precision) : precision_(precision) {
  if (precision != FPP_PREC_FP64 && precision != FPP_PREC_MIXED)
    throw std::runtime_error("precision must be FPP_PREC_FP64 or FPP_PREC_MIXED");
}

PairFLAREGB300::~PairFLAREGB300() {
  if (model_) fpp_model_destroy(model_);
  if (b2_) fpp_b2_destroy(b2_);
}

void PairFLAREGB300::read_file(const std::string &filename) {
  parse_file(filename);
  if (model_) fpp_model_destroy(model_);
  if (b2_) fpp_b2_destroy(b2_);
  model_ = nullptr;
  b2_ = nullptr;
  const double radial_hyps[2] = {0.0, cutoff};
  const int32_t settings[3] = {n_species, n_max, l_max};
  check(fpp_b2_create(radial_string.c_str(), cutoff_string.c_str(), radial_hyps, 2, nullptr,
                      0, settings, cutoffs.data(), &b2_),
        "fpp_b2_create");
  check(fpp_model_create(b2_, 1.0, (double)power, &model_), "fpp_model_create");
  check(fpp_model_set_beta(model_, power, beta.data()), "fpp_model_set_beta");
  // MAXMEM (GB) caps the device memory of one compute, as the Kokkos pair
  // style reads it (pair_flare_kokkos.cpp:737-743)
  if (const char *mm = std::getenv("MAXMEM"))
    check(fpp_model_set_max_memory(model_, std::atof(mm) * 1.0e9), "fpp_model_set_max_memory");
}

int PairFLAREGB300::batches() const {
  int32_t n = 0;
  if (model_) check(fpp_model_pair_batches(model_, &n), "fpp_model_pair_batches");
  return n;
}

void PairFLAREGB300::parse_file(const std::string &filename) {
  std::ifstream in(filename);
  if (!in) throw std::runtime_error("Cannot open potential file " + filename);
  std::string line;
  std::getline(in, line);  // date and contributor
  std::getline(in, line);
  {
    std::istringstream ls(line);
    std::string word;
    ls >> word;
    char *end = nullptr;
    const long p = std::strtol(word.c_str(), &end, 10);
    legacy_layout = word.empty() || *end != '\0';
    if (legacy_layout) {
      power = 2;             // older layout: this line is the radial basis
      radial_string = word;
    } else {
      power = (int)p;
      std::getline(in, line);
      std::istringstream rs(line);
      rs >> radial_string;
    }
  }
  std::getline(in, line);
  {
    std::istringstream ls(line);
    ls >> n_species >> n_max >> l_max >> beta_size;
  }
  std::getline(in, line);
  {
    std::istringstream ls(line);
    ls >> cutoff_string;
  }
  if (legacy_layout) {
    const double c = grab(in, 1)[0];
    cutoffs.assign((size_t)n_species * n_species, c);
  } else {
    cutoffs = grab(in, (size_t)n_species * n_species);
  }
  cutoff = -1;
  for (double c : cutoffs) cutoff = c > cutoff ? c : cutoff;
  const int n_radial = n_max * n_species;
  const int n_d = n_radial * (n_radial + 1) / 2 * (l_max + 1);
  int beta_check;
  if (power == 1)
    beta_check = n_d;
  else if (power == 2)
    beta_check = n_d * (n_d + 1) / 2;
  else
    throw std::runtime_error("Power should be 1 or 2.");
  if (beta_check != beta_size)
    throw std::runtime_error("Beta size doesn't match the number of descriptors.");
  beta = grab(in, (size_t)beta_size * n_species);
}

void PairFLAREGB300::compute(int eflag, int vflag, double **x, double **f, const int *type,
                             int nlocal, int nghost, int inum, const int *ilist,
                             const int *numneigh, int *const *firstneigh, double *eng_vdwl,
                             double *virial, double *eatom) {
  if (!model_) throw std::runtime_error("pair flare/gb300: coefficients not read");
  // the full neighbor list, flattened in ilist order
  numneigh_.resize(inum);
  neighbors_.clear();
  for (int ii = 0; ii < inum; ii++) {
    const int i = ilist[ii];
    numneigh_[ii] = numneigh[i];
    neighbors_.insert(neighbors_.end(), firstneigh[i], firstneigh[i] + numneigh[i]);
  }
  const int nall = nlocal + nghost;
  double e = 0, v[6] = {0, 0, 0, 0, 0, 0};
  check(fpp_pair_compute(model_, nlocal, nall, nall ? x[0] : nullptr, type, inum, ilist,
                         numneigh_.data(), neighbors_.data(), precision_,
                         nall ? f[0] : nullptr, &e, v, eatom, nullptr),
        "fpp_pair_compute");
  if (eflag && eng_vdwl) *eng_vdwl += e;
  if (vflag && virial)
    for (int k = 0; k < 6; k++) virial[k] += v[k];
}
