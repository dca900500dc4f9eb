/* Spin-orbital (T) restated in C - TEST INFRASTRUCTURE ONLY (no product code calls it).
 *
 * The formula of oracle/spin_orbital_oracle.py (ExaChem's (T) over spin orbitals,
 * exachem/cc/ccsd_t/ccsd_t_all_fused_cpu.hpp: the contraction families and the energy loop
 * :597-619), per occupied triplet i < j < k, densely over all virtual spin orbitals:
 *
 *   X_p[x][y][z] = - sum_e t2[x][e][j'][k'] v2iabc[i'][e][y][z] - sum_m t2[y][z][i'][m] v2ijka[j'][k'][m][x]
 *   for the permutations p = (i', j', k') in {(i,j,k), (j,i,k), (k,j,i)}
 *   W(abc) = sum_p s_p (X_p[a][b][c] - X_p[b][a][c] - X_p[c][b][a]),  s = (+1, -1, -1)
 *   V(abc) = the same permutations of t1[x][i'] v2ijab[j'][k'][y][z]
 *   E[T] += W W / D,  E(T) += (W + V) W / D  over a < b < c,  D = e_i + e_j + e_k - e_a - e_b - e_c
 *
 * Layouts as ccsdt_energy_spin_orbital takes them (t1[V][O], t2[V][V][O][O], v2ijab[O][O][V][V],
 * v2ijka[O][O][O][V], v2iabc[O][V][V][V]).  No spin blocking: every triplet costs the same
 * 3 V^3 (V + O) multiply-adds, so a timed sample of triplets projects to the whole exactly.
 * OpenMP over the rows x of each X and the first virtual index of the energy; compensated
 * (TwoSum) double sums, one partial per index a, added in a fixed order (the same bits for any
 * thread count). */
#include <stdlib.h>
#include <string.h>

typedef struct {
  double s, c;
} csum;

static void cadd(csum* a, double x) { /* Knuth TwoSum into (s, c) */
  const double t = a->s + x, z = t - a->s;
  a->c += (a->s - (t - z)) + (x - z);
  a->s = t;
}

static void so_x(int O, int V, const double* t2, const double* v2ijka, const double* v2iabc, int ip, int jp, int kp,
                 double* X) {
  const long long V2 = (long long) V * V, O2 = (long long) O * O;
#pragma omp parallel for schedule(static)
  for(int x = 0; x < V; x++) {
    double* row = X + (long long) x * V2;
    memset(row, 0, sizeof(double) * V2);
    for(int e = 0; e < V; e++) { /* d-term */
      const double  c = t2[((long long) x * V + e) * O2 + (long long) jp * O + kp];
      const double* w = v2iabc + ((long long) ip * V + e) * V2;
      if(c != 0.0)
        for(long long yz = 0; yz < V2; yz++) row[yz] -= c * w[yz];
    }
    for(long long yz = 0; yz < V2; yz++) { /* s-term */
      const double* tr = t2 + yz * O2 + (long long) ip * O;
      const double* u  = v2ijka + ((long long) jp * O + kp) * O * V + x;
      double        s  = 0.0;
      for(int m = 0; m < O; m++) s += tr[m] * u[(long long) m * V];
      row[yz] -= s;
    }
  }
}

/* E[T], E(T) of the listed triplets (tri[3 n], each i < j < k; NULL = every triplet).
 * Returns 0, or -1 when a triplet is out of range or the scratch cannot be allocated. */
int so_oracle_energy(int oa, int ob, int va, int vb, const double* eps_o, const double* eps_v, const double* t1,
                     const double* t2, const double* v2ijab, const double* v2ijka, const double* v2iabc, long n,
                     const int* tri, double* e4_out, double* e5_out) {
  const int O = oa + ob, V = va + vb;
  (void) ob;
  (void) vb;
  *e4_out = *e5_out = 0.0;
  if(O < 3 || V < 3) return 0;
  const long long V2 = (long long) V * V, V3 = V2 * V;
  double*         X  = (double*) malloc(sizeof(double) * 3 * V3);
  csum*           pa = (csum*) malloc(sizeof(csum) * 2 * V);
  if(!X || !pa) {
    free(X);
    free(pa);
    return -1;
  }
  csum e4 = {0.0, 0.0}, e5 = {0.0, 0.0};
  const long  all = (long) O * (O - 1) * (O - 2) / 6;
  int         ti = 0, tj = 1, tk = 2;
  for(long q = 0; q < (tri ? n : all); q++) {
    int i, j, k;
    if(tri) {
      i = tri[3 * q], j = tri[3 * q + 1], k = tri[3 * q + 2];
      if(!(0 <= i && i < j && j < k && k < O)) {
        free(X);
        free(pa);
        return -1;
      }
    } else { /* lexicographic enumeration of i < j < k */
      i = ti, j = tj, k = tk;
      if(++tk == O) {
        if(++tj == O - 1) tj = ++ti + 1;
        tk = tj + 1;
      }
    }
    const int perm[3][3] = {{i, j, k}, {j, i, k}, {k, j, i}};
    for(int p = 0; p < 3; p++) so_x(O, V, t2, v2ijka, v2iabc, perm[p][0], perm[p][1], perm[p][2], X + p * V3);
    const double eo = eps_o[i] + eps_o[j] + eps_o[k];
#pragma omp parallel for schedule(dynamic)
    for(int a = 0; a < V; a++) {
      csum* s4 = pa + 2 * a;
      csum* s5 = s4 + 1;
      s4->s = s4->c = s5->s = s5->c = 0.0;
      for(int b = a + 1; b < V; b++)
        for(int c = b + 1; c < V; c++) {
          const int xyz[3][3] = {{a, b, c}, {b, a, c}, {c, b, a}};
          double    w = 0.0, v = 0.0;
          for(int p = 0; p < 3; p++) {
            const double* Xp = X + p * V3;
            for(int r = 0; r < 3; r++) {
              const int    x = xyz[r][0], y = xyz[r][1], z = xyz[r][2];
              const double sg = ((p == 0) == (r == 0)) ? 1.0 : -1.0;
              w += sg * Xp[(long long) x * V2 + (long long) y * V + z];
              v += sg * t1[(long long) x * O + perm[p][0]] *
                   v2ijab[(((long long) perm[p][1] * O + perm[p][2]) * V + y) * V + z];
            }
          }
          const double d = eo - eps_v[a] - eps_v[b] - eps_v[c];
          cadd(s4, w * w / d);
          cadd(s5, (w + v) * w / d);
        }
    }
    for(int a = 0; a < V; a++) {
      cadd(&e4, pa[2 * a].s);
      cadd(&e4, pa[2 * a].c);
      cadd(&e5, pa[2 * a + 1].s);
      cadd(&e5, pa[2 * a + 1].c);
    }
  }
  free(X);
  free(pa);
  *e4_out = e4.s + e4.c;
  *e5_out = e5.s + e5.c;
  return 0;
}
