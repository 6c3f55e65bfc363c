/*
 * CPU oracle in plain C (FP64, OpenMP over atoms).  TEST INFRASTRUCTURE ONLY:
 * used by tests/ as the checker at sizes numpy cannot reach and by bench.py as
 * the timed CPU baseline; the flare_pp_gb300 package never calls it.
 *
 * It restates the mapped-beta pair style of mir-group/flare_pp on a periodic
 * structure, atom by atom as the reference does:
 *   - neighbors: Structure::compute_neighbors (src/flare_pp/structure.cpp:
 *     52-118) semantics -- wrapped positions (:120-133), image shifts in
 *     [-sweep, sweep]^3 with sweep = ceil(cutoff / single_sweep_cutoff),
 *     dist < cutoff && dist != 0; found here through fractional-coordinate
 *     bins instead of the O(N^2) scan (same pair set);
 *   - per atom: single_bond_multiple_cutoffs, B2_descriptor and
 *     compute_energy_and_u (lammps_plugins/lammps_descriptor.cpp:7-304) with
 *     the B2 filter r <= cutoffs[s_i][s_j] (src/flare_pp/descriptors/
 *     b2.cpp:277), E_i = p^T beta p / |p|^2 as a per-atom GEMV
 *     (pair_flare.cpp:95-136), skipped when |p|^2 < 1e-8;
 *   - pair forces f_ij = u . d c / d r_ij added to atom i and subtracted from
 *     j (pair_flare.cpp:141-175); the stress is -(1/V) sum f_a r_b in the
 *     order xx, xy, xz, yy, yz, zz.
 * B3 (oracle_b3_beta_form, below) follows the same per-atom form.
 * Radial basis: chebyshev x quadratic cutoff (radial.cpp:138-169, cutoffs.cpp:
 * 44-56).  Harmonics: the solid-harmonic recurrence of oracle/basis.py, which
 * tests pin against the reference's y_grad.cpp.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXL 8
#define PI_ 3.14159265358979323846

static double g_norm[(MAXL + 1) * (MAXL + 1)];
static double g_dfact[MAXL + 1];

static void init_tables(void) {
  static int done = 0;
  if (done) return;
  for (int l = 0; l <= MAXL; l++)
    for (int m = 0; m <= MAXL; m++) {
      double v = 0;
      if (m <= l) {
        double f = 1;
        for (int k = l - m + 1; k <= l + m; k++) f *= k;
        v = sqrt((2 * l + 1) / (4 * PI_) / f);
        if (m > 0) v *= sqrt(2.0);
      }
      g_norm[l * (MAXL + 1) + m] = v;
    }
  for (int m = 0; m <= MAXL; m++) {
    double d = 1;
    for (int k = 1; k < 2 * m; k += 2) d *= k;
    g_dfact[m] = d;
  }
  done = 1;
}

/* Y[lm], dY[3*lm + k] */
static void harmonics(double x, double y, double z, int lmax, double *Y, double *dY) {
  const double r = sqrt(x * x + y * y + z * z), ir = 1.0 / r;
  const double ux = x * ir, uy = y * ir, uz = z * ir;
  double A = 1, B = 0, Ap = 1, Bp = 0;
  for (int m = 0; m <= lmax; m++) {
    if (m > 0) {
      Ap = A;
      Bp = B;
      double a2 = ux * A - uy * B, b2 = uy * A + ux * B;
      A = a2;
      B = b2;
    }
    const double Ax = m * Ap, Ay = -m * Bp, Bx = m * Bp, By = m * Ap;
    double q1 = 0, q2 = 0, z1 = 0, z2 = 0, r1 = 0, r2 = 0;
    for (int l = m; l <= lmax; l++) {
      double q, qz, qr;
      if (l == m) {
        q = g_dfact[m];
        qz = 0;
        qr = 0;
      } else if (l == m + 1) {
        q = (2 * m + 1) * uz * q1;
        qz = (2 * m + 1) * q1;
        qr = 0;
      } else {
        const double a = 2 * l - 1, b = l + m - 1, inv = 1.0 / (l - m);
        q = (a * uz * q1 - b * q2) * inv;
        qz = (a * (q1 + uz * z1) - b * z2) * inv;
        qr = (a * uz * r1 - b * (q2 + r2)) * inv;
      }
      q2 = q1;
      q1 = q;
      z2 = z1;
      z1 = qz;
      r2 = r1;
      r1 = qr;
      const double nrm = g_norm[l * (MAXL + 1) + m];
      int ip = l * l + l + m;
      double R = nrm * q * A;
      Y[ip] = R;
      dY[3 * ip + 0] = (nrm * (qr * 2 * ux * A + q * Ax) - l * R * ux) * ir;
      dY[3 * ip + 1] = (nrm * (qr * 2 * uy * A + q * Ay) - l * R * uy) * ir;
      dY[3 * ip + 2] = (nrm * (qz + qr * 2 * uz) * A - l * R * uz) * ir;
      if (m > 0) {
        int im = l * l + l - m;
        double S = nrm * q * B;
        Y[im] = S;
        dY[3 * im + 0] = (nrm * (qr * 2 * ux * B + q * Bx) - l * S * ux) * ir;
        dY[3 * im + 1] = (nrm * (qr * 2 * uy * B + q * By) - l * S * uy) * ir;
        dY[3 * im + 2] = (nrm * (qz + qr * 2 * uz) * B - l * S * uz) * ir;
      }
    }
  }
}

/* g_n, dg_n/dr of chebyshev x quadratic cutoff (radial.cpp:138-169) */
static void radial(double r, double r1, double rc, int N, double *g, double *dg) {
  double fc = 0, dfc = 0;
  if (r <= rc) {
    double d = r - rc;
    fc = d * d;
    dfc = 2 * d;
  }
  int inside = !(r < r1 || r > rc);
  double c = 1.0 / (rc - r1), x = (r - r1) * c;
  double t2 = 0, t1 = 0, d2 = 0, d1 = 0;
  for (int n = 0; n < N; n++) {
    double t, dt;
    if (n == 0) {
      t = 1;
      dt = 0;
    } else if (n == 1) {
      t = x;
      dt = c;
    } else {
      t = 2 * x * t1 - t2;
      dt = 2 * t1 * c + 2 * x * d1 - d2;
    }
    t2 = t1;
    t1 = t;
    d2 = d1;
    d1 = dt;
    if (!inside) {
      t = 0;
      dt = 0;
    }
    g[n] = t * fc;
    dg[n] = dt * fc + t * dfc;
  }
}

static void inv3(const double *a, double *o) {
  double c00 = a[4] * a[8] - a[5] * a[7];
  double c01 = a[5] * a[6] - a[3] * a[8];
  double c02 = a[3] * a[7] - a[4] * a[6];
  double det = a[0] * c00 + a[1] * c01 + a[2] * c02;
  o[0] = c00 / det;
  o[3] = c01 / det;
  o[6] = c02 / det;
  o[1] = (a[2] * a[7] - a[1] * a[8]) / det;
  o[4] = (a[0] * a[8] - a[2] * a[6]) / det;
  o[7] = (a[1] * a[6] - a[0] * a[7]) / det;
  o[2] = (a[1] * a[5] - a[2] * a[4]) / det;
  o[5] = (a[2] * a[3] - a[0] * a[5]) / det;
  o[8] = (a[0] * a[4] - a[1] * a[3]) / det;
}

static void mm3(const double *a, const double *m, double *o) {
  for (int j = 0; j < 3; j++)
    o[j] = (a[0] * m[0 * 3 + j] + a[1] * m[1 * 3 + j]) + a[2] * m[2 * 3 + j];
}

static double dot3(const double *a, const double *b) {
  return (a[0] * b[0] + a[1] * b[1]) + a[2] * b[2];
}

typedef struct {
  int noa, sweep, ns_img, nb[3];
  double cell[9], cutoff, delta[3], volume;
  double *wp, *frac;
  int *bin_start, *bin_atoms;
} Geo;

static int geo_init(Geo *G, int noa, const double *cell, const double *pos, double cutoff) {
  memset(G, 0, sizeof(*G));
  G->noa = noa;
  memcpy(G->cell, cell, 9 * sizeof(double));
  G->cutoff = cutoff;
  double ct[9], cti[9], cd[9], cdi[9];
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) ct[i * 3 + j] = cell[j * 3 + i];
  inv3(ct, cti);
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++)
      cd[i * 3 + j] = (cell[i * 3] * ct[j] + cell[i * 3 + 1] * ct[3 + j]) + cell[i * 3 + 2] * ct[6 + j];
  inv3(cd, cdi);
  double c00 = cell[4] * cell[8] - cell[5] * cell[7];
  double c01 = cell[5] * cell[6] - cell[3] * cell[8];
  double c02 = cell[3] * cell[7] - cell[4] * cell[6];
  G->volume = fabs(cell[0] * c00 + cell[1] * c01 + cell[2] * c02);
  const double *v1 = cell, *v2 = cell + 3, *v3 = cell + 6;
  double ab = dot3(v1, v2), ac = dot3(v1, v3), bc = dot3(v2, v3);
  double a = sqrt(dot3(v1, v1)), b = sqrt(dot3(v2, v2)), c = sqrt(dot3(v3, v3));
#define HH(x, cs) ((x) * sqrt(1 - (cs) * (cs)))
  double cand[6] = {HH(a, ab / (a * b)), HH(b, ab / (a * b)), HH(a, ac / (a * c)),
                    HH(c, ac / (a * c)), HH(b, bc / (b * c)), HH(c, bc / (b * c))};
  double ssc = cand[0];
  for (int k = 0; k < 6; k++)
    if (cand[k] < ssc) ssc = cand[k];
  G->sweep = (int)ceil(cutoff / ssc);
  G->ns_img = 2 * G->sweep + 1;
  double margin = 1e-6 * (1 + cutoff);
  for (int k = 0; k < 3; k++) {
    const double *p = cell + 3 * ((k + 1) % 3), *q = cell + 3 * ((k + 2) % 3);
    double cx = p[1] * q[2] - p[2] * q[1], cy = p[2] * q[0] - p[0] * q[2],
           cz = p[0] * q[1] - p[1] * q[0];
    double h = G->volume / sqrt(cx * cx + cy * cy + cz * cz);
    int nb = (int)floor(h / (cutoff * (1 + 1e-6) + 1e-6));
    G->nb[k] = nb < 1 ? 1 : (nb > 512 ? 512 : nb);
    G->delta[k] = (cutoff + margin) / h + 1e-9;
  }
  int nbins = G->nb[0] * G->nb[1] * G->nb[2];
  G->wp = (double *)malloc(sizeof(double) * 3 * (noa ? noa : 1));
  G->frac = (double *)malloc(sizeof(double) * 3 * (noa ? noa : 1));
  G->bin_start = (int *)calloc(nbins + 1, sizeof(int));
  G->bin_atoms = (int *)malloc(sizeof(int) * (noa ? noa : 1));
  int *bin_of = (int *)malloc(sizeof(int) * (noa ? noa : 1));
  if (!G->wp || !G->frac || !G->bin_start || !G->bin_atoms || !bin_of) return -1;
  for (int i = 0; i < noa; i++) {
    double t[3], rel[3], rw[3], w[3];
    mm3(pos + 3 * i, ct, t);
    mm3(t, cdi, rel);
    for (int k = 0; k < 3; k++) rw[k] = rel[k] - floor(rel[k]);
    mm3(rw, cd, t);
    mm3(t, cti, w);
    for (int k = 0; k < 3; k++) {
      G->wp[3 * i + k] = w[k];
      G->frac[3 * i + k] = rw[k];
    }
    int bk[3];
    for (int k = 0; k < 3; k++) {
      int v = (int)floor(rw[k] * G->nb[k]);
      bk[k] = v < 0 ? 0 : (v >= G->nb[k] ? G->nb[k] - 1 : v);
    }
    bin_of[i] = (bk[0] * G->nb[1] + bk[1]) * G->nb[2] + bk[2];
    G->bin_start[bin_of[i] + 1]++;
  }
  for (int b = 0; b < nbins; b++) G->bin_start[b + 1] += G->bin_start[b];
  int *cur = (int *)calloc(nbins, sizeof(int));
  for (int i = 0; i < noa; i++) G->bin_atoms[G->bin_start[bin_of[i]] + cur[bin_of[i]]++] = i;
  free(cur);
  free(bin_of);
  return 0;
}

static void geo_free(Geo *G) {
  free(G->wp);
  free(G->frac);
  free(G->bin_start);
  free(G->bin_atoms);
}

/* neighbors of atom i: (j, x, y, z, r); returns count (<= cap) */
static int neighbors_of(const Geo *G, int i, int cap, int *js, double *rel) {
  int n = 0;
  const double *wi = G->wp + 3 * i, *fi = G->frac + 3 * i;
  for (int s1 = -G->sweep; s1 <= G->sweep; s1++)
    for (int s2 = -G->sweep; s2 <= G->sweep; s2++)
      for (int s3 = -G->sweep; s3 <= G->sweep; s3++) {
        int sv[3] = {s1, s2, s3}, lo[3], hi[3], empty = 0;
        for (int k = 0; k < 3; k++) {
          double c = fi[k] - sv[k];
          int l = (int)floor((c - G->delta[k]) * G->nb[k]);
          int h = (int)floor((c + G->delta[k]) * G->nb[k]);
          lo[k] = l < 0 ? 0 : l;
          hi[k] = h > G->nb[k] - 1 ? G->nb[k] - 1 : h;
          if (lo[k] > hi[k]) empty = 1;
        }
        if (empty) continue;
        for (int b0 = lo[0]; b0 <= hi[0]; b0++)
          for (int b1 = lo[1]; b1 <= hi[1]; b1++)
            for (int b2 = lo[2]; b2 <= hi[2]; b2++) {
              int bin = (b0 * G->nb[1] + b1) * G->nb[2] + b2;
              for (int t = G->bin_start[bin]; t < G->bin_start[bin + 1]; t++) {
                int j = G->bin_atoms[t];
                const double *wj = G->wp + 3 * j;
                double im[3];
                for (int k = 0; k < 3; k++) {
                  double v = (wj[k] - wi[k]) + s1 * G->cell[k];
                  v = v + s2 * G->cell[3 + k];
                  im[k] = v + s3 * G->cell[6 + k];
                }
                double d = sqrt((im[0] * im[0] + im[1] * im[1]) + im[2] * im[2]);
                if (d < G->cutoff && d != 0) {
                  if (n < cap) {
                    js[n] = j;
                    rel[4 * n] = im[0];
                    rel[4 * n + 1] = im[1];
                    rel[4 * n + 2] = im[2];
                    rel[4 * n + 3] = d;
                  }
                  n++;
                }
              }
            }
      }
  return n;
}

/*
 * Mapped-beta energy, forces and stress (power 1 or 2).
 * beta: n_species dense n_d x n_d matrices (power 2) or n_species vectors
 * (power 1).  atoms/n_atoms: the atoms to evaluate (NULL = all); forces
 * accumulate the contributions of the evaluated atoms only.
 * Returns 0, or -1 on allocation failure / -2 when an atom has more than
 * 4096 neighbors.
 */
int oracle_beta_form(int noa, const double *cell, const int *species, const double *pos,
                     int n_species, int N, int lmax, double r1, const double *cutoffs,
                     const double *beta, int power, const int *atoms, int n_atoms,
                     int n_threads, double *energy, double *forces, double *stress,
                     double *atom_e) {
  init_tables();
  double cmax = 0;
  for (int k = 0; k < n_species * n_species; k++)
    if (cutoffs[k] > cmax) cmax = cutoffs[k];
  Geo G;
  if (geo_init(&G, noa, cell, pos, cmax)) return -1;
  const int H = (lmax + 1) * (lmax + 1), nr = n_species * N, sb = nr * H;
  const int L1 = lmax + 1, nd = nr * (nr + 1) / 2 * L1;
  const int cap = 4096;
  int na = atoms ? n_atoms : noa;
  int err = 0;
  double etot = 0, vir[9] = {0};
  memset(forces, 0, sizeof(double) * 3 * noa);
  if (atom_e) memset(atom_e, 0, sizeof(double) * noa);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel
  {
    int *js = (int *)malloc(sizeof(int) * cap);
    double *rel = (double *)malloc(sizeof(double) * 4 * cap);
    double *bas = (double *)malloc(sizeof(double) * (size_t)cap * (2 * N + 4 * H));
    double *c = (double *)malloc(sizeof(double) * sb);
    double *u = (double *)malloc(sizeof(double) * sb);
    double *p = (double *)malloc(sizeof(double) * nd);
    double *bp = (double *)malloc(sizeof(double) * nd);
    double *w = (double *)malloc(sizeof(double) * nd);
    double *F = (double *)calloc(3 * (size_t)noa, sizeof(double));
    double lvir[9] = {0}, le = 0;
    int lerr = (!js || !rel || !bas || !c || !u || !p || !bp || !w || !F) ? -1 : 0;
#pragma omp for schedule(dynamic, 16)
    for (int ii = 0; ii < na; ii++) {
      if (lerr) continue;
      int i = atoms ? atoms[ii] : ii;
      int si = species[i];
      int nn = neighbors_of(&G, i, cap, js, rel);
      if (nn > cap) {
        lerr = -2;
        continue;
      }
      memset(c, 0, sizeof(double) * sb);
      int keep_n = 0;
      for (int q = 0; q < nn; q++) {
        int sj = species[js[q]];
        double rc = cutoffs[si * n_species + sj];
        double r = rel[4 * q + 3];
        if (!(r <= rc)) {
          js[q] = -1;
          continue;
        }
        double *b = bas + (size_t)q * (2 * N + 4 * H);
        radial(r, r1, rc, N, b, b + N);
        harmonics(rel[4 * q], rel[4 * q + 1], rel[4 * q + 2], lmax, b + 2 * N, b + 2 * N + H);
        for (int n = 0; n < N; n++)
          for (int lm = 0; lm < H; lm++) c[(sj * N + n) * H + lm] += b[n] * b[2 * N + lm];
        keep_n++;
      }
      (void)keep_n;
      int d = 0;
      double nsq = 0;
      for (int n1 = 0; n1 < nr; n1++)
        for (int n2 = n1; n2 < nr; n2++)
          for (int l = 0; l < L1; l++, d++) {
            double v = 0;
            for (int m = 0; m < 2 * l + 1; m++)
              v += c[n1 * H + l * l + m] * c[n2 * H + l * l + m];
            p[d] = v;
            nsq += v * v;
          }
      if (nsq < 1e-8) continue;
      const double *Bm = beta + (size_t)si * (power == 2 ? (size_t)nd * nd : (size_t)nd);
      double e = 0;
      if (power == 2) {
        for (int a = 0; a < nd; a++) {
          const double *row = Bm + (size_t)a * nd;
          double s = 0;
          for (int k = 0; k < nd; k++) s += row[k] * p[k];
          bp[a] = s;
        }
        for (int a = 0; a < nd; a++) e += p[a] * bp[a];
        e /= nsq;
        for (int a = 0; a < nd; a++) w[a] = 2 * (bp[a] - e * p[a]) / nsq;
      } else {
        double nr_ = sqrt(nsq);
        for (int a = 0; a < nd; a++) e += p[a] * Bm[a];
        e /= nr_;
        for (int a = 0; a < nd; a++) w[a] = Bm[a] / nr_ - e * p[a] / nsq;
      }
      le += e;
      if (atom_e) atom_e[i] = e;
      /* u = dE/dc (lammps_descriptor.cpp:272-303) */
      memset(u, 0, sizeof(double) * sb);
      for (int n1 = 0; n1 < nr; n1++)
        for (int n2 = 0; n2 < nr; n2++) {
          int lo = n1 < n2 ? n1 : n2, hi = n1 < n2 ? n2 : n1;
          int q = lo * nr - lo * (lo - 1) / 2 + (hi - lo);
          double fac = n1 == n2 ? 2.0 : 1.0;
          for (int l = 0; l < L1; l++) {
            double wv = fac * w[q * L1 + l];
            for (int m = 0; m < 2 * l + 1; m++)
              u[n1 * H + l * l + m] += wv * c[n2 * H + l * l + m];
          }
        }
      for (int q = 0; q < nn; q++) {
        if (js[q] < 0) continue;
        int j = js[q], sj = species[j];
        const double *b = bas + (size_t)q * (2 * N + 4 * H);
        double r = rel[4 * q + 3];
        double ux = rel[4 * q] / r, uy = rel[4 * q + 1] / r, uz = rel[4 * q + 2] / r;
        double f[3] = {0, 0, 0};
        for (int n = 0; n < N; n++)
          for (int lm = 0; lm < H; lm++) {
            double uv = u[(sj * N + n) * H + lm];
            double rad = b[N + n] * b[2 * N + lm];
            f[0] += uv * (rad * ux + b[n] * b[2 * N + H + 3 * lm]);
            f[1] += uv * (rad * uy + b[n] * b[2 * N + H + 3 * lm + 1]);
            f[2] += uv * (rad * uz + b[n] * b[2 * N + H + 3 * lm + 2]);
          }
        for (int k = 0; k < 3; k++) {
          F[3 * i + k] += f[k];
          F[3 * j + k] -= f[k];
          for (int k2 = 0; k2 < 3; k2++) lvir[3 * k + k2] += f[k] * rel[4 * q + k2];
        }
      }
    }
#pragma omp critical
    {
      if (lerr) err = lerr;
      etot += le;
      for (int k = 0; k < 9; k++) vir[k] += lvir[k];
      if (F)
        for (int k = 0; k < 3 * noa; k++) forces[k] += F[k];
    }
    free(js);
    free(rel);
    free(bas);
    free(c);
    free(u);
    free(p);
    free(bp);
    free(w);
    free(F);
  }
  *energy = etot;
  double vi = 1.0 / G.volume;
  stress[0] = -vir[0] * vi;
  stress[1] = -vir[1] * vi;
  stress[2] = -vir[2] * vi;
  stress[3] = -vir[4] * vi;
  stress[4] = -vir[5] * vi;
  stress[5] = -vir[8] * vi;
  geo_free(&G);
  return err;
}

/*
 * B2 descriptors of every atom (the values of B2::compute_struc,
 * src/flare_pp/descriptors/b2.cpp:181-242 and :244-399, without the stored
 * derivatives), in atom order: p (noa x n_d, the n1 <= n2, l order of
 * b2.cpp:205-218) and |p|.  Same neighbors, filter and bases as
 * oracle_beta_form.  Returns 0, -1 (allocation) or -2 (more than 4096
 * neighbors).
 */
int oracle_b2_descriptors(int noa, const double *cell, const int *species, const double *pos,
                          int n_species, int N, int lmax, double r1, const double *cutoffs,
                          int n_threads, double *p_out, double *norms) {
  init_tables();
  double cmax = 0;
  for (int k = 0; k < n_species * n_species; k++)
    if (cutoffs[k] > cmax) cmax = cutoffs[k];
  Geo G;
  if (geo_init(&G, noa, cell, pos, cmax)) return -1;
  const int H = (lmax + 1) * (lmax + 1), nr = n_species * N, sb = nr * H;
  const int L1 = lmax + 1, nd = nr * (nr + 1) / 2 * L1;
  const int cap = 4096;
  int err = 0;
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel
  {
    int *js = (int *)malloc(sizeof(int) * cap);
    double *rel = (double *)malloc(sizeof(double) * 4 * cap);
    double *b = (double *)malloc(sizeof(double) * (2 * N + 4 * H));
    double *c = (double *)malloc(sizeof(double) * sb);
    int lerr = (!js || !rel || !b || !c) ? -1 : 0;
#pragma omp for schedule(dynamic, 16)
    for (int i = 0; i < noa; i++) {
      if (lerr) continue;
      int si = species[i];
      int nn = neighbors_of(&G, i, cap, js, rel);
      if (nn > cap) {
        lerr = -2;
        continue;
      }
      memset(c, 0, sizeof(double) * sb);
      for (int q = 0; q < nn; q++) {
        int sj = species[js[q]];
        double rc = cutoffs[si * n_species + sj];
        double r = rel[4 * q + 3];
        if (!(r <= rc)) continue;
        radial(r, r1, rc, N, b, b + N);
        harmonics(rel[4 * q], rel[4 * q + 1], rel[4 * q + 2], lmax, b + 2 * N, b + 2 * N + H);
        for (int n = 0; n < N; n++)
          for (int lm = 0; lm < H; lm++) c[(sj * N + n) * H + lm] += b[n] * b[2 * N + lm];
      }
      double *p = p_out + (size_t)i * nd;
      int d = 0;
      double nsq = 0;
      for (int n1 = 0; n1 < nr; n1++)
        for (int n2 = n1; n2 < nr; n2++)
          for (int l = 0; l < L1; l++, d++) {
            double v = 0;
            for (int m = 0; m < 2 * l + 1; m++)
              v += c[n1 * H + l * l + m] * c[n2 * H + l * l + m];
            p[d] = v;
            nsq += v * v;
          }
      norms[i] = sqrt(nsq);
    }
#pragma omp critical
    {
      if (lerr) err = lerr;
    }
    free(js);
    free(rel);
    free(b);
    free(c);
  }
  geo_free(&G);
  return err;
}

/*
 * B3 (src/flare_pp/descriptors/b3.cpp:134-382) in the same per-atom form:
 * complex single bond from the real one (c[l,+m] = (-1)^m (R + iS)/sqrt2,
 * c[l,-m] = (R - iS)/sqrt2 with R = c_real[l,m], S = c_real[l,-m]), the
 * bispectrum over n1 <= n2 <= n3 and triangles (l1,l2,l3), E_i and w as for
 * B2, u = dE/dc (holomorphic) mapped back to dE/dc_real, then the B2 pair
 * forces.  Coefficients: Wigner 3j by Racah's formula, with the entries that
 * the reference's lmax = 4 table holds as 0 (non-integer rationals written
 * there as integer divisions, descriptors/wigner3j.cpp:590-1986).
 */
static double fact_(int n) {
  double f = 1;
  for (int k = 2; k <= n; k++) f *= k;
  return f;
}

static double w3j_(int l1, int l2, int l3, int m1, int m2, int m3) {
  if (m1 + m2 + m3 != 0 || l3 < abs(l1 - l2) || l3 > l1 + l2) return 0;
  if (abs(m1) > l1 || abs(m2) > l2 || abs(m3) > l3) return 0;
  double pre = fact_(l1 + l2 - l3) * fact_(l1 - l2 + l3) * fact_(-l1 + l2 + l3) /
               fact_(l1 + l2 + l3 + 1) * fact_(l1 + m1) * fact_(l1 - m1) * fact_(l2 + m2) *
               fact_(l2 - m2) * fact_(l3 + m3) * fact_(l3 - m3);
  int kmin = 0, kmax = l1 + l2 - l3;
  if (l2 - l3 - m1 > kmin) kmin = l2 - l3 - m1;
  if (l1 - l3 + m2 > kmin) kmin = l1 - l3 + m2;
  if (l1 - m1 < kmax) kmax = l1 - m1;
  if (l2 + m2 < kmax) kmax = l2 + m2;
  double s = 0;
  for (int k = kmin; k <= kmax; k++)
    s += ((k & 1) ? -1.0 : 1.0) /
         (fact_(k) * fact_(l3 - l2 + k + m1) * fact_(l3 - l1 + k - m2) *
          fact_(l1 + l2 - l3 - k) * fact_(l1 - k - m1) * fact_(l2 - k + m2));
  double w = (((l1 - l2 - m3) % 2) ? -1.0 : 1.0) * sqrt(pre) * s;
  return w;
}

static double b3_coeff_(int l1, int l2, int l3, int m1, int m2, int m3, int lmax) {
  double w = w3j_(l1, l2, l3, m1, m2, m3);
  if (lmax == 4 && w != 0 && fabs(w) < 1) {
    double inv2 = 1 / (w * w), k = floor(sqrt(inv2) + 0.5);
    if (k > 1 && fabs(inv2 - k * k) < 1e-9 * inv2) return 0;
  }
  return w;
}

typedef struct {
  int n_ls, n_terms;
  int beg[70];
  int i1[1500], i2[1500], i3[1500];
  double w[1500];
} B3T;

static void b3_tables_(int lmax, B3T *T) {
  int t = 0, e = 0;
  for (int l1 = 0; l1 <= lmax; l1++)
    for (int l2 = 0; l2 <= lmax; l2++)
      for (int l3 = 0; l3 <= lmax; l3++) {
        if (abs(l1 - l2) > l3 || l3 > l1 + l2) continue;
        T->beg[t++] = e;
        for (int m1 = -l1; m1 <= l1; m1++)
          for (int m2 = -l2; m2 <= l2; m2++) {
            int m3 = -m1 - m2;
            if (abs(m3) > l3) continue;
            double w = b3_coeff_(l1, l2, l3, m1, m2, m3, lmax);
            if (w == 0) continue;
            T->i1[e] = l1 * l1 + l1 + m1;
            T->i2[e] = l2 * l2 + l2 + m2;
            T->i3[e] = l3 * l3 + l3 + m3;
            T->w[e] = w;
            e++;
          }
      }
  T->beg[t] = e;
  T->n_ls = t;
  T->n_terms = e;
}

/* real c (nr x H) -> complex (re, im) */
static void to_complex_(const double *c, int nr, int lmax, double *zr, double *zi) {
  const int H = (lmax + 1) * (lmax + 1);
  const double is2 = 0.70710678118654752440;
  for (int n = 0; n < nr; n++)
    for (int l = 0; l <= lmax; l++) {
      const double *cl = c + n * H + l * l + l;
      double *r = zr + n * H + l * l + l, *im = zi + n * H + l * l + l;
      r[0] = cl[0];
      im[0] = 0;
      for (int m = 1; m <= l; m++) {
        double sg = (m & 1) ? -1 : 1, R = cl[m], S = cl[-m];
        r[m] = sg * R * is2;
        im[m] = sg * S * is2;
        r[-m] = R * is2;
        im[-m] = -S * is2;
      }
    }
}

int oracle_b3_beta_form(int noa, const double *cell, const int *species, const double *pos,
                        int n_species, int N, int lmax, double r1, double rcut,
                        const double *beta, int power, const int *atoms, int n_atoms,
                        int n_threads, double *energy, double *forces, double *stress,
                        double *atom_e) {
  init_tables();
  if (lmax > 4 || n_species * N > 64) return -3;
  B3T *T = (B3T *)malloc(sizeof(B3T));
  if (!T) return -1;
  b3_tables_(lmax, T);
  Geo G;
  if (geo_init(&G, noa, cell, pos, rcut)) {
    free(T);
    return -1;
  }
  const int H = (lmax + 1) * (lmax + 1), nr = n_species * N, sb = nr * H;
  const int ntri = nr * (nr + 1) * (nr + 2) / 6, nls = T->n_ls, nd = ntri * nls;
  int *tri = (int *)malloc(sizeof(int) * 3 * ntri);
  {
    int k = 0;
    for (int a = 0; a < nr; a++)
      for (int b = a; b < nr; b++)
        for (int c = b; c < nr; c++, k++) {
          tri[3 * k] = a;
          tri[3 * k + 1] = b;
          tri[3 * k + 2] = c;
        }
  }
  const int cap = 4096;
  int na = atoms ? n_atoms : noa;
  int err = 0;
  double etot = 0, vir[9] = {0};
  memset(forces, 0, sizeof(double) * 3 * noa);
  if (atom_e) memset(atom_e, 0, sizeof(double) * noa);
#ifdef _OPENMP
  if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
#pragma omp parallel
  {
    int *js = (int *)malloc(sizeof(int) * cap);
    double *rel = (double *)malloc(sizeof(double) * 4 * cap);
    double *bas = (double *)malloc(sizeof(double) * (size_t)cap * (2 * N + 4 * H));
    double *c = (double *)malloc(sizeof(double) * sb);
    double *zr = (double *)malloc(sizeof(double) * sb);
    double *zi = (double *)malloc(sizeof(double) * sb);
    double *ur = (double *)malloc(sizeof(double) * sb);
    double *ui = (double *)malloc(sizeof(double) * sb);
    double *u = (double *)malloc(sizeof(double) * sb);
    double *p = (double *)malloc(sizeof(double) * nd);
    double *bp = (double *)malloc(sizeof(double) * nd);
    double *w = (double *)malloc(sizeof(double) * nd);
    double *F = (double *)calloc(3 * (size_t)noa, sizeof(double));
    double lvir[9] = {0}, le = 0;
    int lerr = (!js || !rel || !bas || !c || !zr || !zi || !ur || !ui || !u || !p || !bp ||
                !w || !F || !tri)
                   ? -1
                   : 0;
#pragma omp for schedule(dynamic, 16)
    for (int ii = 0; ii < na; ii++) {
      if (lerr) continue;
      int i = atoms ? atoms[ii] : ii;
      int si = species[i];
      int nn = neighbors_of(&G, i, cap, js, rel);
      if (nn > cap) {
        lerr = -2;
        continue;
      }
      memset(c, 0, sizeof(double) * sb);
      for (int q = 0; q < nn; q++) {
        int sj = species[js[q]];
        double r = rel[4 * q + 3];
        if (!(r <= rcut)) {  /* b3.cpp:258 */
          js[q] = -1;
          continue;
        }
        double *b = bas + (size_t)q * (2 * N + 4 * H);
        radial(r, r1, rcut, N, b, b + N);
        harmonics(rel[4 * q], rel[4 * q + 1], rel[4 * q + 2], lmax, b + 2 * N, b + 2 * N + H);
        for (int n = 0; n < N; n++)
          for (int lm = 0; lm < H; lm++) c[(sj * N + n) * H + lm] += b[n] * b[2 * N + lm];
      }
      to_complex_(c, nr, lmax, zr, zi);
      double nsq = 0;
      for (int r = 0; r < ntri; r++) {
        const double *a1r = zr + tri[3 * r] * H, *a1i = zi + tri[3 * r] * H;
        const double *a2r = zr + tri[3 * r + 1] * H, *a2i = zi + tri[3 * r + 1] * H;
        const double *a3r = zr + tri[3 * r + 2] * H, *a3i = zi + tri[3 * r + 2] * H;
        for (int t = 0; t < nls; t++) {
          double v = 0;
          for (int e = T->beg[t]; e < T->beg[t + 1]; e++) {
            int x1 = T->i1[e], x2 = T->i2[e], x3 = T->i3[e];
            double xr = a1r[x1] * a2r[x2] - a1i[x1] * a2i[x2];
            double xi = a1r[x1] * a2i[x2] + a1i[x1] * a2r[x2];
            v += T->w[e] * (xr * a3r[x3] - xi * a3i[x3]);
          }
          p[r * nls + t] = v;
          nsq += v * v;
        }
      }
      if (nsq < 1e-8) continue;
      const double *Bm = beta + (size_t)si * (power == 2 ? (size_t)nd * nd : (size_t)nd);
      double e = 0;
      if (power == 2) {
        for (int a = 0; a < nd; a++) {
          const double *row = Bm + (size_t)a * nd;
          double s = 0;
          for (int k = 0; k < nd; k++) s += row[k] * p[k];
          bp[a] = s;
        }
        for (int a = 0; a < nd; a++) e += p[a] * bp[a];
        e /= nsq;
        for (int a = 0; a < nd; a++) w[a] = 2 * (bp[a] - e * p[a]) / nsq;
      } else {
        double nr_ = sqrt(nsq);
        for (int a = 0; a < nd; a++) e += p[a] * Bm[a];
        e /= nr_;
        for (int a = 0; a < nd; a++) w[a] = Bm[a] / nr_ - e * p[a] / nsq;
      }
      le += e;
      if (atom_e) atom_e[i] = e;
      /* u = dE/dc (complex), then dE/dc_real */
      memset(ur, 0, sizeof(double) * sb);
      memset(ui, 0, sizeof(double) * sb);
      for (int r = 0; r < ntri; r++) {
        int n1 = tri[3 * r], n2 = tri[3 * r + 1], n3 = tri[3 * r + 2];
        for (int t = 0; t < nls; t++) {
          double wq = w[r * nls + t];
          for (int ee = T->beg[t]; ee < T->beg[t + 1]; ee++) {
            int k1 = n1 * H + T->i1[ee], k2 = n2 * H + T->i2[ee], k3 = n3 * H + T->i3[ee];
            double f = wq * T->w[ee];
            double ar = zr[k1], ai = zi[k1], br = zr[k2], bi = zi[k2], cr = zr[k3], ci = zi[k3];
            ur[k1] += f * (br * cr - bi * ci);
            ui[k1] += f * (br * ci + bi * cr);
            ur[k2] += f * (ar * cr - ai * ci);
            ui[k2] += f * (ar * ci + ai * cr);
            ur[k3] += f * (ar * br - ai * bi);
            ui[k3] += f * (ar * bi + ai * br);
          }
        }
      }
      {
        const double is2 = 0.70710678118654752440;
        for (int n = 0; n < nr; n++)
          for (int l = 0; l <= lmax; l++) {
            int o = n * H + l * l + l;
            u[o] = ur[o];
            for (int m = 1; m <= l; m++) {
              double sg = (m & 1) ? -1 : 1;
              u[o + m] = (sg * ur[o + m] + ur[o - m]) * is2;
              u[o - m] = (ui[o - m] - sg * ui[o + m]) * is2;
            }
          }
      }
      for (int q = 0; q < nn; q++) {
        if (js[q] < 0) continue;
        int j = js[q], sj = species[j];
        const double *b = bas + (size_t)q * (2 * N + 4 * H);
        double r = rel[4 * q + 3];
        double ux = rel[4 * q] / r, uy = rel[4 * q + 1] / r, uz = rel[4 * q + 2] / r;
        double f[3] = {0, 0, 0};
        for (int n = 0; n < N; n++)
          for (int lm = 0; lm < H; lm++) {
            double uv = u[(sj * N + n) * H + lm];
            double rad = b[N + n] * b[2 * N + lm];
            f[0] += uv * (rad * ux + b[n] * b[2 * N + H + 3 * lm]);
            f[1] += uv * (rad * uy + b[n] * b[2 * N + H + 3 * lm + 1]);
            f[2] += uv * (rad * uz + b[n] * b[2 * N + H + 3 * lm + 2]);
          }
        for (int k = 0; k < 3; k++) {
          F[3 * i + k] += f[k];
          F[3 * j + k] -= f[k];
          for (int k2 = 0; k2 < 3; k2++) lvir[3 * k + k2] += f[k] * rel[4 * q + k2];
        }
      }
    }
#pragma omp critical
    {
      if (lerr) err = lerr;
      etot += le;
      for (int k = 0; k < 9; k++) vir[k] += lvir[k];
      if (F)
        for (int k = 0; k < 3 * noa; k++) forces[k] += F[k];
    }
    free(js);
    free(rel);
    free(bas);
    free(c);
    free(zr);
    free(zi);
    free(ur);
    free(ui);
    free(u);
    free(p);
    free(bp);
    free(w);
    free(F);
  }
  *energy = etot;
  double vi = 1.0 / G.volume;
  stress[0] = -vir[0] * vi;
  stress[1] = -vir[1] * vi;
  stress[2] = -vir[2] * vi;
  stress[3] = -vir[4] * vi;
  stress[4] = -vir[5] * vi;
  stress[5] = -vir[8] * vi;
  geo_free(&G);
  free(tri);
  free(T);
  return err;
}

int oracle_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
