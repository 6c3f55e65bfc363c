// A LAMMPS-shaped driver of PairFLAREGB300 (flare_pp_gb300/lammps): builds
// the arrays LAMMPS hands a pair style -- x and f as contiguous rows behind
// double**, 1-based type, ilist / numneigh / firstneigh of a full neighbor
// list -- from a case file, calls read_file and compute(eflag = vflag = 1),
// and writes energy, virial, forces and per-atom energies.
//
//   pair_harness --parse-only potential.txt       header fields, no GPU calls
//   pair_harness potential.txt case.txt out.txt [fp64|mixed]
//
// case.txt: "nlocal nghost inum", then nall rows of x, nall types, inum
// ilist entries, nlocal numneigh (indexed by atom), then each listed atom's
// neighbors in ilist order.
#include <cstdio>
#include <fstream>
#include <iostream>
#include <stdexcept>
#include <vector>

#include "pair_flare_gb300.h"

int main(int argc, char **argv) {
  try {
    if (argc == 3 && std::string(argv[1]) == "--parse-only") {
      PairFLAREGB300 p;
      p.parse_file(argv[2]);
      std::printf("power %d radial %s n_species %d n_max %d l_max %d beta_size %d "
                  "cutoff_function %s cutoff %.6f legacy %d n_beta %zu\n",
                  p.power, p.radial_string.c_str(), p.n_species, p.n_max, p.l_max,
                  p.beta_size, p.cutoff_string.c_str(), p.cutoff, (int)p.legacy_layout,
                  p.beta.size());
      return 0;
    }
    if (argc < 4) {
      std::fprintf(stderr, "usage: pair_harness potential case out [fp64|mixed]\n");
      return 2;
    }
    const bool fp64 = argc > 4 && std::string(argv[4]) == "fp64";
    std::ifstream in(argv[2]);
    int nlocal, nghost, inum;
    in >> nlocal >> nghost >> inum;
    const int nall = nlocal + nghost;
    std::vector<double> xs((size_t)nall * 3), fs((size_t)nall * 3, 0.0), eatom(nall, 0.0);
    for (auto &v : xs) in >> v;
    std::vector<int> type(nall), ilist(inum), numneigh(nlocal);
    for (auto &v : type) in >> v;
    for (auto &v : ilist) in >> v;
    for (auto &v : numneigh) in >> v;
    std::vector<std::vector<int>> lists(nlocal);
    for (int ii = 0; ii < inum; ii++) {
      const int i = ilist[ii];
      lists[i].resize(numneigh[i]);
      for (auto &v : lists[i]) in >> v;
    }
    if (!in) throw std::runtime_error("bad case file");
    std::vector<double *> x(nall), f(nall);
    std::vector<int *> firstneigh(nlocal);
    for (int k = 0; k < nall; k++) {
      x[k] = xs.data() + 3 * k;
      f[k] = fs.data() + 3 * k;
    }
    for (int i = 0; i < nlocal; i++) firstneigh[i] = lists[i].data();
    PairFLAREGB300 pair(fp64 ? FPP_PREC_FP64 : FPP_PREC_MIXED);
    pair.read_file(argv[1]);
    double eng = 0, virial[6] = {0, 0, 0, 0, 0, 0};
    pair.compute(1, 1, x.data(), f.data(), type.data(), nlocal, nghost, inum, ilist.data(),
                 numneigh.data(), firstneigh.data(), &eng, virial, eatom.data());
    std::FILE *out = std::fopen(argv[3], "w");
    std::fprintf(out, "%.17g %d\n", eng, pair.batches());
    for (double v : virial) std::fprintf(out, "%.17g ", v);
    std::fprintf(out, "\n");
    for (int k = 0; k < nall; k++)
      std::fprintf(out, "%.17g %.17g %.17g %.17g\n", fs[3 * k], fs[3 * k + 1], fs[3 * k + 2],
                   eatom[k]);
    std::fclose(out);
    return 0;
  } catch (const std::exception &e) {
    std::fprintf(stderr, "pair_harness: %s\n", e.what());
    return 1;
  }
}
