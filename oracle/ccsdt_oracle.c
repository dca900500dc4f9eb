/*
 * CPU oracle for the closed-shell (T) energy.  TEST INFRASTRUCTURE ONLY: it is the
 * checker for the CUDA path (tests/, __graft_entry__.smoke(), bench.py's CPU
 * baseline) and is never linked into or called by the product library.
 *
 * It restates, in spatial orbitals, what ExaChem's fused (T) computes in spin
 * orbitals (exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp:20-631, driven by the task
 * loop of ccsd_t_fused_driver.hpp:368-483).  The reference forms per tile block
 *   t3d = 9 d1 + 9 d2 contractions (cpu.hpp:172-270, 330-428),
 *   t3s = 9 s1 contractions        (cpu.hpp:472-577),
 *   E[T] += f t3d^2 / D,  E(T) += f t3d (t3d + t3s) / D,
 *   D = e_h1 + e_h2 + e_h3 - e_p4 - e_p5 - e_p6   (cpu.hpp:597-619),
 * with f = 2 (restricted) / symmetry factors (ccsd_t_fused_driver.hpp:387-395).
 * Summed over the closed-shell spin cases this equals, per occupied triplet
 * i <= j <= k with multiplicity m (6 distinct, 3 two equal, 1 all equal):
 *
 *   X(ia,jb,kc) = sum_d t_ij^ad (kc|bd) - sum_l t_il^ab (jl|kc)
 *   W_abc       = X(ia,jb,kc) + X(ia,kc,jb) + X(jb,ia,kc) + X(jb,kc,ia) + X(kc,ia,jb) + X(kc,jb,ia)
 *   V_abc       = W_abc + (jb|kc) t_i^a + (ia|kc) t_j^b + (ia|jb) t_k^c
 *   Z_abc       = 4 W_abc + W_bca + W_cab
 *   Y_abc       = 3 V_abc - V_acb - V_bac - V_cba   (W in place of V for E[T])
 *   E(T)_ijk    = m/9 sum_abc Z_abc Y_abc / D_ijk^abc
 *
 * (the full-space form (1/3) sum_{ijk,abc} Z (V_abc - V_cba) / D summed over the six
 * orderings of (i,j,k): reordering the occupied indices conjugates the a<->c swap into
 * each of the three transpositions twice, which gives Y).
 *
 * The d2 family (contracted virtual p7, cpu.hpp:330-428) is the sum over d, the d1
 * family (contracted occupied h7, cpu.hpp:172-270) the sum over l, s1 (cpu.hpp:472-577)
 * the t1 terms of V.  The equivalence is checked numerically against the reference
 * itself (oracle/_ref, built from the unmodified reference headers) in the tests.
 *
 * Layouts (row-major): eps_occ[o], eps_vir[v], t1[o][v], t2[o][o][v][v] = t_ij^ab,
 * oovv[o][o][v][v] = (ia|jb), ooov[o][o][o][v] = (ij|ka), ovvv[o][v][v][v] = (ia|bc).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  int                  o, v;
  const double *       eo, *ev, *t1, *t2, *oovv, *ooov;
  const double* const* slab; /* slab[z] = ovvv + z v^3 (only the triplet's z are read) */
} sys_t;

/* Neumaier compensated accumulation */
typedef struct {
  double s, c;
} csum_t;
static inline void cs_add(csum_t* a, double x) {
  double t = a->s + x;
  if(fabs(a->s) >= fabs(x)) a->c += (a->s - t) + x;
  else a->c += (x - t) + a->s;
  a->s = t;
}

/* W[a][b][c] += sum_d t_xy^{alpha d} (z gamma|beta d) - sum_l t_xl^{alpha beta} (yl|z gamma)
 * for one of the six pair orderings; (alpha, beta, gamma) are the virtual indices that
 * pair with (x, y, z).  pos[] maps (alpha, beta, gamma) to the W slots (a, b, c). */
static void add_perm_rows(const sys_t* S, double* W, int x, int y, int z, const int pos[3], int a0, int a1) {
  const int     o = S->o, v = S->v;
  const size_t  v2 = (size_t) v * v;
  const double* T   = S->t2 + ((size_t) x * o + y) * v2; /* T[alpha][d] */
  const double* I   = S->slab[z];                        /* I[gamma][beta][d] */
  const size_t  st[3] = {v2, (size_t) v, 1};
  const size_t  sa = st[pos[0]], sb = st[pos[1]], sc = st[pos[2]];
#pragma omp parallel for schedule(static)
  for(int al = a0; al < a1; al++) {
    double* hol = (double*) malloc(sizeof(double) * (size_t) o * v); /* hol[l][gamma] = (yl|z gamma) */
    for(int l = 0; l < o; l++)
      for(int ga = 0; ga < v; ga++)
        hol[(size_t) l * v + ga] = S->ooov[(((size_t) y * o + l) * o + z) * v + ga];
    const double* Ta = T + (size_t) al * v;
    for(int be = 0; be < v; be++) {
      double tl[512];
      int    nl = o <= 512 ? o : 512;
      for(int l = 0; l < nl; l++) tl[l] = S->t2[(((size_t) x * o + l) * v + al) * v + be];
      for(int ga = 0; ga < v; ga++) {
        const double* Ig = I + ((size_t) ga * v + be) * v;
        double        acc = 0.0;
        for(int d = 0; d < v; d++) acc += Ta[d] * Ig[d];
        double h = 0.0;
        for(int l = 0; l < o; l++) {
          double tv = l < nl ? tl[l] : S->t2[(((size_t) x * o + l) * v + al) * v + be];
          h += tv * hol[(size_t) l * v + ga];
        }
        W[al * sa + be * sb + ga * sc] += acc - h;
      }
    }
    free(hol);
  }
}
static void add_perm(const sys_t* S, double* W, int x, int y, int z, const int pos[3]) {
  add_perm_rows(S, W, x, y, z, pos, 0, S->v);
}

/* W for one ordered triplet (i, j, k): sum of the six pair orderings */
static void build_w(const sys_t* S, double* W, int i, int j, int k) {
  const int p_abc[3] = {0, 1, 2}; /* X(ia,jb,kc): alpha=a beta=b gamma=c */
  const int p_acb[3] = {0, 2, 1}; /* X(ia,kc,jb): alpha=a beta=c gamma=b */
  const int p_bac[3] = {1, 0, 2}; /* X(jb,ia,kc) */
  const int p_bca[3] = {1, 2, 0}; /* X(jb,kc,ia) */
  const int p_cab[3] = {2, 0, 1}; /* X(kc,ia,jb) */
  const int p_cba[3] = {2, 1, 0}; /* X(kc,jb,ia) */
  memset(W, 0, sizeof(double) * (size_t) S->v * S->v * S->v);
  add_perm(S, W, i, j, k, p_abc);
  add_perm(S, W, i, k, j, p_acb);
  add_perm(S, W, j, i, k, p_bac);
  add_perm(S, W, j, k, i, p_bca);
  add_perm(S, W, k, i, j, p_cab);
  add_perm(S, W, k, j, i, p_cba);
}

static int multiplicity(int i, int j, int k) {
  if(i == j && j == k) return 1;
  if(i == j || j == k || i == k) return 3;
  return 6;
}

/* energy of one triplet from its W (cpu.hpp:597-619 restated) */
static void triplet_energy(const sys_t* S, const double* W, int i, int j, int k, double* e4,
                           double* e5) {
  const int    o = S->o, v = S->v;
  const size_t v2 = (size_t) v * v;
  const double eijk = S->eo[i] + S->eo[j] + S->eo[k];
  const double* oovv = S->oovv;
  const double* t1 = S->t1;
  csum_t        s4 = {0, 0}, s5 = {0, 0};
#pragma omp parallel
  {
    csum_t l4 = {0, 0}, l5 = {0, 0};
#pragma omp for schedule(static)
    for(int a = 0; a < v; a++)
      for(int b = 0; b < v; b++)
        for(int c = 0; c < v; c++) {
          double wabc = W[a * v2 + b * v + c], wbca = W[b * v2 + c * v + a];
          double wcab = W[c * v2 + a * v + b], wacb = W[a * v2 + c * v + b];
          double wbac = W[b * v2 + a * v + c], wcba = W[c * v2 + b * v + a];
          double z    = 4.0 * wabc + wbca + wcab;
          double y4   = 3.0 * wabc - wacb - wbac - wcba;
          /* singles part of V_xyz: (jy|kz) t_i^x + (ix|kz) t_j^y + (ix|jy) t_k^z */
#define SGL(X, Y, Z)                                                                     \
  (oovv[((size_t) j * o + k) * v2 + (Y) * v + (Z)] * t1[(size_t) i * v + (X)] +          \
   oovv[((size_t) i * o + k) * v2 + (X) * v + (Z)] * t1[(size_t) j * v + (Y)] +          \
   oovv[((size_t) i * o + j) * v2 + (X) * v + (Y)] * t1[(size_t) k * v + (Z)])
          double y5 = y4 + 3.0 * SGL(a, b, c) - SGL(a, c, b) - SGL(b, a, c) - SGL(c, b, a);
#undef SGL
          double d = eijk - S->ev[a] - S->ev[b] - S->ev[c];
          cs_add(&l4, z * y4 / d);
          cs_add(&l5, z * y5 / d);
        }
#pragma omp critical
    {
      cs_add(&s4, l4.s);
      cs_add(&s4, l4.c);
      cs_add(&s5, l5.s);
      cs_add(&s5, l5.c);
    }
  }
  double m = multiplicity(i, j, k) / 9.0;
  *e4      = m * (s4.s + s4.c);
  *e5      = m * (s5.s + s5.c);
}

int oracle_triplets_slabs(int o, int v, const double* eo, const double* ev, const double* t1,
                          const double* t2, const double* oovv, const double* ooov,
                          const double* const* slab, long n, const int* tri, double* out4,
                          double* out5);

/* Per-triplet energies for a list of triplets (tri[3 n], each i <= j <= k).
 * out4 / out5 receive E[T] / E(T) contributions; returns 0 or an error code. */
int oracle_triplets(int o, int v, const double* eo, const double* ev, const double* t1,
                    const double* t2, const double* oovv, const double* ooov, const double* ovvv,
                    long n, const int* tri, double* out4, double* out5) {
  if(o <= 0 || v <= 0) return 1;
  const double** slab = (const double**) malloc(sizeof(double*) * (size_t) o);
  if(!slab) return 2;
  for(int z = 0; z < o; z++) slab[z] = ovvv + (size_t) z * v * v * v;
  int rc = oracle_triplets_slabs(o, v, eo, ev, t1, t2, oovv, ooov, slab, n, tri, out4, out5);
  free(slab);
  return rc;
}

/* As oracle_triplets, with the (ia|bc) integrals given as one v^3 slab per occupied i
 * (slab[i] may be NULL for any i that no listed triplet contains). */
int oracle_triplets_slabs(int o, int v, const double* eo, const double* ev, const double* t1,
                          const double* t2, const double* oovv, const double* ooov,
                          const double* const* slab, long n, const int* tri, double* out4,
                          double* out5) {
  if(o <= 0 || v <= 0) return 1;
  sys_t   S = {o, v, eo, ev, t1, t2, oovv, ooov, slab};
  double* W = (double*) malloc(sizeof(double) * (size_t) v * v * v);
  if(!W) return 2;
  for(long t = 0; t < n; t++) {
    int i = tri[3 * t], j = tri[3 * t + 1], k = tri[3 * t + 2];
    if(!(0 <= i && i <= j && j <= k && k < o) || !slab[i] || !slab[j] || !slab[k]) {
      free(W);
      return 3;
    }
    build_w(&S, W, i, j, k);
    triplet_energy(&S, W, i, j, k, &out4[t], &out5[t]);
  }
  free(W);
  return 0;
}

/* Full (T): every triplet i <= j <= k, compensated total. */
int oracle_energy(int o, int v, const double* eo, const double* ev, const double* t1,
                  const double* t2, const double* oovv, const double* ooov, const double* ovvv,
                  double* e4, double* e5) {
  long n = (long) o * (o + 1) * (o + 2) / 6;
  int* tri = (int*) malloc(sizeof(int) * 3 * (size_t) (n > 0 ? n : 1));
  double *p4 = (double*) malloc(sizeof(double) * (size_t) (n > 0 ? n : 1)),
         *p5 = (double*) malloc(sizeof(double) * (size_t) (n > 0 ? n : 1));
  long t = 0;
  for(int i = 0; i < o; i++)
    for(int j = i; j < o; j++)
      for(int k = j; k < o; k++) {
        tri[3 * t] = i;
        tri[3 * t + 1] = j;
        tri[3 * t + 2] = k;
        t++;
      }
  int rc = oracle_triplets(o, v, eo, ev, t1, t2, oovv, ooov, ovvv, n, tri, p4, p5);
  csum_t s4 = {0, 0}, s5 = {0, 0};
  for(long q = 0; q < n && rc == 0; q++) {
    cs_add(&s4, p4[q]);
    cs_add(&s5, p5[q]);
  }
  *e4 = s4.s + s4.c;
  *e5 = s5.s + s5.c;
  free(tri);
  free(p4);
  free(p5);
  return rc;
}

int oracle_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/* Timing sample for the CPU baseline: the six pair orderings of triplet (i, j, k) restricted to
 * the first-virtual rows alpha in [a0, a1), i.e. (a1 - a0) / v of the triplet's contraction
 * multiply-adds (which are all but O(v^3) of its work), into a scratch W that is then discarded.
 * slab as in oracle_triplets_slabs.  Returns 0 or an error code. */
int oracle_w_rows_sample(int o, int v, const double* eo, const double* ev, const double* t1,
                         const double* t2, const double* oovv, const double* ooov,
                         const double* const* slab, int i, int j, int k, int a0, int a1) {
  if(o <= 0 || v <= 0 || a0 < 0 || a1 > v || a0 > a1) return 1;
  if(!(0 <= i && i <= j && j <= k && k < o) || !slab[i] || !slab[j] || !slab[k]) return 3;
  sys_t   S = {o, v, eo, ev, t1, t2, oovv, ooov, slab};
  double* W = (double*) calloc((size_t) v * v * v, sizeof(double));
  if(!W) return 2;
  const int p[6][3] = {{0, 1, 2}, {0, 2, 1}, {1, 0, 2}, {1, 2, 0}, {2, 0, 1}, {2, 1, 0}};
  const int x[6] = {i, i, j, j, k, k}, y[6] = {j, k, i, k, i, j}, z[6] = {k, j, k, i, j, i};
  for(int q = 0; q < 6; q++) add_perm_rows(&S, W, x[q], y[q], z[q], p[q], a0, a1);
  free(W);
  return 0;
}
