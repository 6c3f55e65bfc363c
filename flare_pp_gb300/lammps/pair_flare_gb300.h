// pair_style flare on GB300: the compute of PairFLARE
// (lammps_plugins/pair_flare.h:20-50, pair_flare.cpp:68-184) in one call to
// libflare_pp_gb300 (fpp_pair_compute), as a LAMMPS-independent C++ core.
//
// A LAMMPS pair style derives from LAMMPS_NS::Pair, registers
// PairStyle(flare/gb300, ...) and forwards:
//   coeff(narg, arg)      -> read_file(arg[2])
//   compute(eflag, vflag) -> compute(eflag, vflag, atom->x, atom->f, atom->type,
//                                    atom->nlocal, atom->nghost, list->inum,
//                                    list->ilist, list->numneigh,
//                                    list->firstneigh, &eng_vdwl, virial,
//                                    eflag_atom ? eatom : nullptr)
// with newton_pair on and a full neighbor list, as PairFLARE::init_style
// requires (pair_flare.cpp:238-247).  The MAXMEM environment variable (GB)
// caps the device memory of a compute, as for the Kokkos pair style.  Errors
// are thrown as std::runtime_error (the pair style turns them into
// error->one).
#pragma once

#include <string>
#include <vector>

#include "flare_pp_gb300.h"

class PairFLAREGB300 {
 public:
  explicit PairFLAREGB300(int precision = FPP_PREC_MIXED);
  ~PairFLAREGB300();
  PairFLAREGB300(const PairFLAREGB300 &) = delete;
  PairFLAREGB300 &operator=(const PairFLAREGB300 &) = delete;

  // PairFLARE::read_file (pair_flare.cpp:263-396): the mapped-beta potential
  // file, in the current layout (a power line, n_species^2 cutoffs) or the
  // older one (no power line, power 2, one cutoff for every species pair).
  // Creates the descriptor and model handles and loads beta.
  void read_file(const std::string &filename);
  // The parsing half of read_file alone (host only, no device calls).
  void parse_file(const std::string &filename);

  // PairFLARE::compute (pair_flare.cpp:68-184).  x, f: per-atom rows of 3
  // doubles for the nlocal + nghost atoms, stored contiguously (LAMMPS's
  // memory->create layout); type 1-based.  Forces are added to f;
  // *eng_vdwl and virial[6] (xx, yy, zz, xy, xz, yz) are added to when eflag /
  // vflag are set; eatom (nall, optional) is added to.
  void compute(int eflag, int vflag, double **x, double **f, const int *type, int nlocal,
               int nghost, int inum, const int *ilist, const int *numneigh,
               int *const *firstneigh, double *eng_vdwl, double *virial, double *eatom);

  // Atom batches of the last compute (more than one under a MAXMEM cap).
  int batches() const;

  // Parsed potential (pair_flare.h:30-45 names).
  int power = 0, n_species = 0, n_max = 0, l_max = 0, beta_size = 0;
  std::string radial_string, cutoff_string;
  std::vector<double> cutoffs;  // n_species x n_species, row-major
  double cutoff = 0;            // the largest entry (the neighbor cutoff)
  std::vector<double> beta;     // n_species x beta_size, the file's packed layout
  bool legacy_layout = false;

 private:
  int precision_;
  fpp_b2 *b2_ = nullptr;
  fpp_model *model_ = nullptr;
  std::vector<int32_t> numneigh_, neighbors_;
};
