/*
 * pq_oracle.c -- CPU oracle (test infrastructure only) for the polyquant CI path.
 *
 * A plain-C restatement of the reference algorithms; each function names the
 * reference file:line it follows (paths inside the polyquant project).  The
 * product library never links or calls this file: only tests/, the smoke check
 * and the CPU-baseline leg of bench.py load it, as the checker.
 *
 * Deliberate, result-neutral differences from the reference:
 *   - the determinant hash map + linear det_idx_unfold
 *     (determinant_creation.cpp:378-388) are replaced by an unfold array and
 *     prefix-row addressing that return the same indices;
 *   - the doubles-map skip `unique_dets[..][0][0] < 2`
 *     (determinant_creation.cpp:306) is not reproduced: it only ever fires
 *     wrongly (multi-word strings), for one-word strings it coincides with
 *     "fewer than two particles", where the doubles list is empty anyway.
 */
#include "pq_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXW 8 /* up to 511 orbitals per species in the oracle */

struct orc_detset {
  orc_desc d;
  int n_words;
  int n_spin_blocks[2];
  int64_t n_str[2][2];
  uint64_t *str[2][2];
  int32_t *lvl[2][2];
  int64_t n_dets;
  int32_t *unfold; /* n_dets x ntup */
  int ntup;
  /* addressing */
  int32_t *rowoff0, *rowlen0; /* over species-0 alpha strings */
  int64_t n_e;                /* number of species-0 (alpha,beta) pairs kept */
  int64_t *ebase;             /* n_e */
  int32_t *elev;              /* n_e, allowed species-1 level or -1 */
  int lcap;
  int32_t *prowoff[64], *prowlen[64]; /* per allowed level */
  /* excitation maps (CSR) */
  int64_t *s1_off[2][2];
  int32_t *s1_idx[2][2];
  int64_t *s2_off[2][2];
  int32_t *s2_idx[2][2];
  double *diag;
};

/* ------------------------------------------------------------------------- */
/* integral index helpers: integral.hpp:14-20 (symmetric_matrix_triangular_idx) */
int orc_idx2(int i, int j) { return (i > j) ? (i * (i + 1)) / 2 + j : (j * (j + 1)) / 2 + i; }

static inline double h1v(const orc_detset *ds, int part, int spin, int i, int j) {
  int n = ds->d.n_orb[part];
  return ds->d.h1[part][spin][(int64_t)i + (int64_t)j * n];
}
/* mo_two_body_ints[a][sa][b][sb](row, col), Eigen column-major */
static inline double eriv(const orc_detset *ds, int a, int sa, int b, int sb, int row, int col) {
  int na = ds->d.n_orb[a];
  int64_t npa = (int64_t)na * (na + 1) / 2;
  return ds->d.eri[a][sa][b][sb][(int64_t)row + (int64_t)col * npa];
}
static inline int beta_idx(const orc_detset *ds, int part) { return 1 % ds->n_spin_blocks[part]; }

/* ------------------------------------------------------------------------- */
/* determinant_operations.cpp:4-11 */
int orc_single_spin_num_excitation(const uint64_t *Di, const uint64_t *Dj, int n_words) {
  int deg = 0;
  for (int i = 0; i < n_words; i++) deg += __builtin_popcountll(Di[i] ^ Dj[i]);
  return deg / 2;
}

static int cmp_int(const void *a, const void *b) {
  int x = *(const int *)a, y = *(const int *)b;
  return (x > y) - (x < y);
}

/* determinant_operations.cpp:17-30; orbital index (n_words-1-word)*64 + bit */
int orc_get_holes(const uint64_t *Di, const uint64_t *Dj, int n_words, int *holes) {
  int n = 0;
  for (int i = 0; i < n_words; i++) {
    uint64_t H = (Di[i] ^ Dj[i]) & Di[i];
    while (H) {
      int pos = __builtin_ctzll(H);
      holes[n++] = (n_words - i - 1) * 64 + pos;
      H &= ~(1ULL << pos);
    }
  }
  qsort(holes, n, sizeof(int), cmp_int);
  return n;
}

/* determinant_operations.cpp:32-45 */
int orc_get_parts(const uint64_t *Di, const uint64_t *Dj, int n_words, int *parts) {
  int n = 0;
  for (int i = 0; i < n_words; i++) {
    uint64_t P = (Di[i] ^ Dj[i]) & Dj[i];
    while (P) {
      int pos = __builtin_ctzll(P);
      parts[n++] = (n_words - i - 1) * 64 + pos;
      P &= ~(1ULL << pos);
    }
  }
  qsort(parts, n, sizeof(int), cmp_int);
  return n;
}

/* determinant_operations.cpp:47-116: for each (hole, particle) pair count the
 * occupied orbitals of D_I strictly between them; for doubles add one more
 * permutation when the two ranges interleave (a < c < b < d). */
double orc_get_phase(const uint64_t *Di, const uint64_t *Dj, int n_words, const int *holes, const int *parts, int n_exc) {
  (void)Dj;
  uint64_t nperm = 0;
  for (int l = 0; l < n_exc; l++) {
    uint64_t high = (uint64_t)(parts[l] > holes[l] ? parts[l] : holes[l]);
    uint64_t low = (uint64_t)(parts[l] < holes[l] ? parts[l] : holes[l]) + 1;
    int64_t j = (int64_t)(low >> 6);
    int64_t k = (int64_t)(high >> 6);
    j = n_words - j - 1;
    k = n_words - k - 1;
    uint64_t m = high & 63ULL;
    uint64_t n = low & 63ULL;
    if (j == k) {
      nperm += (uint64_t)__builtin_popcountll(Di[j] & (((1ULL << m) - 1ULL) & (~(1ULL << n) + 1ULL)));
    } else {
      nperm += (uint64_t)__builtin_popcountll(Di[j] & (~0ULL & (~(1ULL << n) + 1ULL)));
      nperm += (uint64_t)__builtin_popcountll(Di[k] & ((1ULL << m) - 1ULL));
      for (int64_t i = k + 1; i < j; i++) nperm += (uint64_t)__builtin_popcountll(Di[i]);
    }
  }
  if (n_exc == 2) {
    int a = holes[0] < parts[0] ? holes[0] : parts[0];
    int b = holes[0] < parts[0] ? parts[0] : holes[0];
    int c = holes[1] < parts[1] ? holes[1] : parts[1];
    int d = holes[1] < parts[1] ? parts[1] : holes[1];
    if (a < c && c < b && b < d) nperm++;
  }
  return (nperm & 1) ? -1.0 : 1.0;
}

/* determinant_operations.cpp:118-137 */
int orc_get_occ_virt(const uint64_t *D, int n_words, int max_orb, int *occ, int *n_occ, int *virt, int *n_virt) {
  int no = 0, nv = 0;
  for (int i = 0; i < n_words; i++) {
    for (int j = 0; j < 64; j++) {
      int orb = (n_words - i - 1) * 64 + j;
      if (orb >= max_orb) break;
      if ((D[i] >> j) & 1ULL)
        occ[no++] = orb;
      else
        virt[nv++] = orb;
    }
  }
  qsort(occ, no, sizeof(int), cmp_int);
  qsort(virt, nv, sizeof(int), cmp_int);
  *n_occ = no;
  *n_virt = nv;
  return 0;
}

/* ------------------------------------------------------------------------- */
/* string enumeration: determinant_creation.cpp:6-42 (create_det),
 * :45-72 (get_unique_excitation_list) and :139-146 (create_unique_excitation);
 * driver order epci.cpp:341-380.  Lexicographic k-combinations of the occupied
 * list (outer) and of the virtual list (inner), as iter::combinations yields. */
static int next_comb(int *c, int k, int n) {
  int i = k - 1;
  while (i >= 0 && c[i] == n - k + i) i--;
  if (i < 0) return 0;
  c[i]++;
  for (int j = i + 1; j < k; j++) c[j] = c[j - 1] + 1;
  return 1;
}

static int64_t make_strings(int n_words, int n_orb, int n_e, int ex_max, uint64_t **out_str, int32_t **out_lvl) {
  int occ[512], virt[512];
  int n_occ = n_e, n_virt = n_orb - n_e;
  for (int i = 0; i < n_occ; i++) occ[i] = i;
  for (int i = 0; i < n_virt; i++) virt[i] = n_e + i;
  /* count */
  int64_t count = 1;
  for (int k = 1; k <= ex_max; k++) {
    if (k > n_virt) return -1; /* "Excitation level exceeds virtual size!" */
    if (k > n_occ) continue;
    double a = 1, b = 1;
    for (int t = 0; t < k; t++) {
      a = a * (n_occ - t) / (t + 1);
      b = b * (n_virt - t) / (t + 1);
    }
    count += (int64_t)llround(a) * (int64_t)llround(b);
  }
  uint64_t *s = (uint64_t *)calloc((size_t)count * n_words, sizeof(uint64_t));
  int32_t *lv = (int32_t *)calloc((size_t)count, sizeof(int32_t));
  uint64_t hf[MAXW] = {0};
  for (int i = 0; i < n_e; i++) hf[n_words - 1 - (i >> 6)] |= 1ULL << (i & 63);
  memcpy(s, hf, sizeof(uint64_t) * n_words);
  lv[0] = 0;
  int64_t pos = 1;
  for (int k = 1; k <= ex_max; k++) {
    if (k > n_occ) continue;
    int co[512], cv[512];
    for (int i = 0; i < k; i++) co[i] = i;
    do {
      for (int i = 0; i < k; i++) cv[i] = i;
      do {
        uint64_t t[MAXW];
        memcpy(t, hf, sizeof(uint64_t) * n_words);
        for (int i = 0; i < k; i++) {
          int o = occ[co[i]];
          t[n_words - 1 - (o >> 6)] &= ~(1ULL << (o & 63));
        }
        for (int i = 0; i < k; i++) {
          int v = virt[cv[i]];
          t[n_words - 1 - (v >> 6)] |= 1ULL << (v & 63);
        }
        memcpy(s + pos * n_words, t, sizeof(uint64_t) * n_words);
        lv[pos] = k;
        pos++;
      } while (next_comb(cv, k, n_virt));
    } while (next_comb(co, k, n_occ));
  }
  *out_str = s;
  *out_lvl = lv;
  return count;
}

/* single/double connectivity maps: determinant_creation.cpp:209-351.  The
 * reference collects, for every string, the indices of listed strings that are
 * one (two) same-spin replacements away, in ascending index order. */
static void make_maps(orc_detset *ds, int part, int spin) {
  int64_t n = ds->n_str[part][spin];
  int nw = ds->n_words;
  const uint64_t *s = ds->str[part][spin];
  int64_t *o1 = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
  int64_t *o2 = (int64_t *)calloc((size_t)n + 1, sizeof(int64_t));
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; i++) {
    int64_t c1 = 0, c2 = 0;
    for (int64_t j = 0; j < n; j++) {
      int e = orc_single_spin_num_excitation(s + i * nw, s + j * nw, nw);
      c1 += (e == 1);
      c2 += (e == 2);
    }
    o1[i + 1] = c1;
    o2[i + 1] = c2;
  }
  for (int64_t i = 0; i < n; i++) {
    o1[i + 1] += o1[i];
    o2[i + 1] += o2[i];
  }
  int32_t *l1 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(o1[n] > 0 ? o1[n] : 1));
  int32_t *l2 = (int32_t *)malloc(sizeof(int32_t) * (size_t)(o2[n] > 0 ? o2[n] : 1));
#pragma omp parallel for schedule(dynamic, 64)
  for (int64_t i = 0; i < n; i++) {
    int64_t p1 = o1[i], p2 = o2[i];
    for (int64_t j = 0; j < n; j++) {
      int e = orc_single_spin_num_excitation(s + i * nw, s + j * nw, nw);
      if (e == 1) l1[p1++] = (int32_t)j;
      if (e == 2) l2[p2++] = (int32_t)j;
    }
  }
  ds->s1_off[part][spin] = o1;
  ds->s1_idx[part][spin] = l1;
  ds->s2_off[part][spin] = o2;
  ds->s2_idx[part][spin] = l2;
}

static inline int str_level(const orc_detset *ds, int part, int spin, int64_t i) { return ds->lvl[part][spin][i]; }

/* prefix length of a spin's string list with level <= L */
static int32_t prefix_le(const orc_detset *ds, int part, int spin, int L) {
  if (L < 0) return 0;
  int64_t n = ds->n_str[part][spin];
  int32_t c = 0;
  while (c < n && ds->lvl[part][spin][c] <= L) c++;
  return c;
}

int64_t orc_lookup(const orc_detset *ds, const int32_t *t) {
  int32_t i = t[0], j = t[1];
  if (i < 0 || j < 0 || i >= ds->n_str[0][0] || j >= ds->n_str[0][1]) return -1;
  if (j >= ds->rowlen0[i]) return -1;
  int64_t ie = (int64_t)ds->rowoff0[i] + j;
  if (ds->d.n_species == 1) return ds->ebase[ie];
  int32_t k = t[2], l = t[3];
  if (k < 0 || l < 0 || k >= ds->n_str[1][0] || l >= ds->n_str[1][1]) return -1;
  int L = ds->elev[ie];
  if (L < 0) return -1;
  if (l >= ds->prowlen[L][k]) return -1;
  return ds->ebase[ie] + ds->prowoff[L][k] + l;
}

/* determinant list: determinant_creation.cpp:148-206 (create_excitation).
 * The excitation degree of a listed string against the HF string equals the
 * level it was generated at, so num_excitation(hf, det) = level sums. */
orc_detset *orc_detset_create(const orc_desc *d, int check_addressing) {
  if (d->n_species < 1 || d->n_species > 2) return NULL;
  orc_detset *ds = (orc_detset *)calloc(1, sizeof(orc_detset));
  ds->d = *d;
  int maxorb = 0;
  for (int s = 0; s < d->n_species; s++) maxorb = d->n_orb[s] > maxorb ? d->n_orb[s] : maxorb;
  ds->n_words = (maxorb >> 6) + 1;
  if (ds->n_words > MAXW) {
    free(ds);
    return NULL;
  }
  for (int s = 0; s < d->n_species; s++) ds->n_spin_blocks[s] = d->restricted[s] ? 1 : 2;
  /* every integral block the element formulas read: h1 per spin block, and
   * (a, sa | b, sb) for b >= a over both species' spin blocks */
  for (int a = 0; a < d->n_species; a++)
    for (int sa = 0; sa < ds->n_spin_blocks[a]; sa++) {
      if (!d->h1[a][sa]) {
        free(ds);
        return NULL;
      }
      for (int b = a; b < d->n_species; b++)
        for (int sb = 0; sb < ds->n_spin_blocks[b]; sb++)
          if (!d->eri[a][sa][b][sb]) {
            free(ds);
            return NULL;
          }
    }
  for (int s = 0; s < d->n_species; s++) {
    int ne[2] = {d->n_alpha[s], d->n_beta[s]};
    for (int sp = 0; sp < 2; sp++) {
      ds->n_str[s][sp] = make_strings(ds->n_words, d->n_orb[s], ne[sp], d->ex_level[s][sp], &ds->str[s][sp], &ds->lvl[s][sp]);
      if (ds->n_str[s][sp] < 0) {
        orc_detset_destroy(ds);
        return NULL;
      }
    }
  }
  int ns = d->n_species;
  ds->ntup = 2 * ns;
  int mc = d->max_collective;
  int tot0 = d->ex_level[0][2];
  /* pass 1: the reference's nested loop order, counting */
  int64_t n0a = ds->n_str[0][0], n0b = ds->n_str[0][1];
  ds->rowoff0 = (int32_t *)calloc((size_t)n0a, sizeof(int32_t));
  ds->rowlen0 = (int32_t *)calloc((size_t)n0a, sizeof(int32_t));
  int64_t ne_tot = 0;
  for (int64_t i = 0; i < n0a; i++) {
    int lim = tot0 - str_level(ds, 0, 0, i);
    if (ns == 1 && mc - str_level(ds, 0, 0, i) < lim) lim = mc - str_level(ds, 0, 0, i);
    ds->rowoff0[i] = (int32_t)ne_tot;
    ds->rowlen0[i] = prefix_le(ds, 0, 1, lim);
    ne_tot += ds->rowlen0[i];
  }
  ds->n_e = ne_tot;
  ds->ebase = (int64_t *)calloc((size_t)(ne_tot + 1), sizeof(int64_t));
  ds->elev = (int32_t *)calloc((size_t)(ne_tot + 1), sizeof(int32_t));
  int64_t psize[64] = {0};
  if (ns == 2) {
    int lmaxa = ds->lvl[1][0][ds->n_str[1][0] - 1], lmaxb = ds->lvl[1][1][ds->n_str[1][1] - 1];
    ds->lcap = lmaxa + lmaxb;
    if (ds->lcap > 63) ds->lcap = 63;
    for (int L = 0; L <= ds->lcap; L++) {
      int64_t n1a = ds->n_str[1][0];
      ds->prowoff[L] = (int32_t *)calloc((size_t)n1a, sizeof(int32_t));
      ds->prowlen[L] = (int32_t *)calloc((size_t)n1a, sizeof(int32_t));
      int64_t acc = 0;
      for (int64_t k = 0; k < n1a; k++) {
        ds->prowoff[L][k] = (int32_t)acc;
        ds->prowlen[L][k] = prefix_le(ds, 1, 1, L - str_level(ds, 1, 0, k));
        acc += ds->prowlen[L][k];
      }
      psize[L] = acc;
    }
  }
  int64_t nd = 0;
  for (int64_t i = 0; i < n0a; i++) {
    for (int32_t j = 0; j < ds->rowlen0[i]; j++) {
      int64_t ie = ds->rowoff0[i] + j;
      ds->ebase[ie] = nd;
      if (ns == 1) {
        ds->elev[ie] = 0;
        nd += 1;
      } else {
        int e0 = str_level(ds, 0, 0, i) + str_level(ds, 0, 1, j);
        int L = d->ex_level[1][2];
        if (mc - e0 < L) L = mc - e0;
        if (L > ds->lcap) L = ds->lcap;
        ds->elev[ie] = L;
        if (L >= 0) nd += psize[L];
      }
    }
  }
  ds->n_dets = nd;
  ds->unfold = (int32_t *)malloc(sizeof(int32_t) * (size_t)(nd > 0 ? nd : 1) * ds->ntup);
  /* pass 2: restate the loop and record unfolded indices in list order */
  int64_t idx = 0;
  for (int64_t i = 0; i < n0a; i++) {
    for (int64_t j = 0; j < n0b; j++) {
      int e0 = str_level(ds, 0, 0, i) + str_level(ds, 0, 1, j);
      if (e0 > tot0) continue;
      if (ns == 1) {
        if (e0 <= mc) {
          ds->unfold[idx * 2 + 0] = (int32_t)i;
          ds->unfold[idx * 2 + 1] = (int32_t)j;
          idx++;
        }
      } else {
        for (int64_t k = 0; k < ds->n_str[1][0]; k++) {
          for (int64_t l = 0; l < ds->n_str[1][1]; l++) {
            int e1 = str_level(ds, 1, 0, k) + str_level(ds, 1, 1, l);
            if (e1 <= d->ex_level[1][2] && e0 + e1 <= mc) {
              int32_t *u = ds->unfold + idx * 4;
              u[0] = (int32_t)i;
              u[1] = (int32_t)j;
              u[2] = (int32_t)k;
              u[3] = (int32_t)l;
              idx++;
            }
          }
        }
      }
    }
  }
  if (idx != nd) {
    fprintf(stderr, "oracle: det count mismatch %lld vs %lld\n", (long long)idx, (long long)nd);
    orc_detset_destroy(ds);
    return NULL;
  }
  if (check_addressing) {
    for (int64_t t = 0; t < nd; t++) {
      if (orc_lookup(ds, ds->unfold + t * ds->ntup) != t) {
        fprintf(stderr, "oracle: addressing mismatch at %lld\n", (long long)t);
        orc_detset_destroy(ds);
        return NULL;
      }
    }
  }
  for (int s = 0; s < ns; s++)
    for (int sp = 0; sp < 2; sp++) make_maps(ds, s, sp);
  return ds;
}

void orc_detset_destroy(orc_detset *ds) {
  if (!ds) return;
  for (int s = 0; s < 2; s++)
    for (int sp = 0; sp < 2; sp++) {
      free(ds->str[s][sp]);
      free(ds->lvl[s][sp]);
      free(ds->s1_off[s][sp]);
      free(ds->s1_idx[s][sp]);
      free(ds->s2_off[s][sp]);
      free(ds->s2_idx[s][sp]);
    }
  for (int L = 0; L < 64; L++) {
    free(ds->prowoff[L]);
    free(ds->prowlen[L]);
  }
  free(ds->rowoff0);
  free(ds->rowlen0);
  free(ds->ebase);
  free(ds->elev);
  free(ds->unfold);
  free(ds->diag);
  free(ds);
}

int orc_n_words(const orc_detset *ds) { return ds->n_words; }
int64_t orc_n_dets(const orc_detset *ds) { return ds->n_dets; }
int64_t orc_n_strings(const orc_detset *ds, int s, int sp) { return ds->n_str[s][sp]; }
const uint64_t *orc_strings(const orc_detset *ds, int s, int sp) { return ds->str[s][sp]; }
const int32_t *orc_unfold(const orc_detset *ds) { return ds->unfold; }
int64_t orc_singles(const orc_detset *ds, int s, int sp, int64_t I, const int32_t **list) {
  *list = ds->s1_idx[s][sp] + ds->s1_off[s][sp][I];
  return ds->s1_off[s][sp][I + 1] - ds->s1_off[s][sp][I];
}
int64_t orc_doubles(const orc_detset *ds, int s, int sp, int64_t I, const int32_t **list) {
  *list = ds->s2_idx[s][sp] + ds->s2_off[s][sp][I];
  return ds->s2_off[s][sp][I + 1] - ds->s2_off[s][sp][I];
}

static inline const uint64_t *getdet(const orc_detset *ds, int part, int spin, int32_t i) {
  return ds->str[part][spin] + (int64_t)i * ds->n_words;
}
static inline int streq(const orc_detset *ds, const uint64_t *a, const uint64_t *b) {
  for (int w = 0; w < ds->n_words; w++)
    if (a[w] != b[w]) return 0;
  return 1;
}

/* ------------------------------------------------------------------------- */
/* slater_condon_singleparticle.cpp:4-51 */
double orc_same_part_ham_diag(const orc_detset *ds, int part, const int32_t *I, const int32_t *J) {
  (void)J;
  const uint64_t *da = getdet(ds, part, 0, I[part * 2 + 0]);
  const uint64_t *db = getdet(ds, part, 1, I[part * 2 + 1]);
  int A = 0, B = beta_idx(ds, part);
  int ao[512], av[512], bo[512], bv[512], nao, nav, nbo, nbv;
  int n = ds->d.n_orb[part];
  orc_get_occ_virt(da, ds->n_words, n, ao, &nao, av, &nav);
  orc_get_occ_virt(db, ds->n_words, n, bo, &nbo, bv, &nbv);
  double e = 0.0;
  for (int x = 0; x < nao; x++) e += h1v(ds, part, A, ao[x], ao[x]);
  for (int x = 0; x < nbo; x++) e += h1v(ds, part, B, bo[x], bo[x]);
  for (int x = 0; x < nao; x++) {
    int i = ao[x];
    for (int y = 0; y < nao; y++) {
      int j = ao[y];
      e += 0.5 * eriv(ds, part, A, part, A, orc_idx2(i, i), orc_idx2(j, j));
      e -= 0.5 * eriv(ds, part, A, part, A, orc_idx2(i, j), orc_idx2(j, i));
    }
    for (int y = 0; y < nbo; y++) {
      int j = bo[y];
      e += 0.5 * eriv(ds, part, A, part, B, orc_idx2(i, i), orc_idx2(j, j));
    }
  }
  for (int x = 0; x < nbo; x++) {
    int i = bo[x];
    for (int y = 0; y < nbo; y++) {
      int j = bo[y];
      e += 0.5 * eriv(ds, part, B, part, B, orc_idx2(i, i), orc_idx2(j, j));
      e -= 0.5 * eriv(ds, part, B, part, B, orc_idx2(i, j), orc_idx2(j, i));
    }
    for (int y = 0; y < nao; y++) {
      int j = ao[y];
      e += 0.5 * eriv(ds, part, B, part, A, orc_idx2(i, i), orc_idx2(j, j));
    }
  }
  return e;
}

/* slater_condon_singleparticle.cpp:53-105 */
double orc_same_part_ham_single(const orc_detset *ds, int part, const int32_t *I, const int32_t *J) {
  const uint64_t *dia = getdet(ds, part, 0, I[part * 2 + 0]);
  const uint64_t *dib = getdet(ds, part, 1, I[part * 2 + 1]);
  const uint64_t *dja = getdet(ds, part, 0, J[part * 2 + 0]);
  const uint64_t *djb = getdet(ds, part, 1, J[part * 2 + 1]);
  int A = 0, B = beta_idx(ds, part);
  int spin = streq(ds, dia, dja) ? 1 : 0;
  int n = ds->d.n_orb[part];
  int ao[512], av[512], bo[512], bv[512], nao, nav, nbo, nbv;
  orc_get_occ_virt(dia, ds->n_words, n, ao, &nao, av, &nav);
  orc_get_occ_virt(dib, ds->n_words, n, bo, &nbo, bv, &nbv);
  int h[4], p[4];
  double e = 0.0;
  if (spin == 0) {
    orc_get_holes(dia, dja, ds->n_words, h);
    orc_get_parts(dia, dja, ds->n_words, p);
    double ph = orc_get_phase(dia, dja, ds->n_words, h, p, 1);
    e += h1v(ds, part, A, h[0], p[0]);
    for (int x = 0; x < nao; x++) {
      int k = ao[x];
      e += eriv(ds, part, A, part, A, orc_idx2(h[0], p[0]), orc_idx2(k, k));
      e -= eriv(ds, part, A, part, A, orc_idx2(h[0], k), orc_idx2(k, p[0]));
    }
    for (int x = 0; x < nbo; x++) {
      int k = bo[x];
      e += eriv(ds, part, A, part, B, orc_idx2(h[0], p[0]), orc_idx2(k, k));
    }
    e *= ph;
  } else {
    orc_get_holes(dib, djb, ds->n_words, h);
    orc_get_parts(dib, djb, ds->n_words, p);
    double ph = orc_get_phase(dib, djb, ds->n_words, h, p, 1);
    e += h1v(ds, part, B, h[0], p[0]);
    for (int x = 0; x < nbo; x++) {
      int k = bo[x];
      e += eriv(ds, part, B, part, B, orc_idx2(h[0], p[0]), orc_idx2(k, k));
      e -= eriv(ds, part, B, part, B, orc_idx2(h[0], k), orc_idx2(k, p[0]));
    }
    for (int x = 0; x < nao; x++) {
      int k = ao[x];
      e += eriv(ds, part, B, part, A, orc_idx2(h[0], p[0]), orc_idx2(k, k));
    }
    e *= ph;
  }
  return e;
}

/* slater_condon_singleparticle.cpp:107-175 */
double orc_same_part_ham_double(const orc_detset *ds, int part, const int32_t *I, const int32_t *J) {
  const uint64_t *dia = getdet(ds, part, 0, I[part * 2 + 0]);
  const uint64_t *dib = getdet(ds, part, 1, I[part * 2 + 1]);
  const uint64_t *dja = getdet(ds, part, 0, J[part * 2 + 0]);
  const uint64_t *djb = getdet(ds, part, 1, J[part * 2 + 1]);
  int A = 0, B = beta_idx(ds, part);
  int nw = ds->n_words;
  double e = 0.0;
  if (streq(ds, dia, dja)) {
    int h[4], p[4];
    orc_get_holes(dib, djb, nw, h);
    orc_get_parts(dib, djb, nw, p);
    double ph = orc_get_phase(dib, djb, nw, h, p, 2);
    e += eriv(ds, part, B, part, B, orc_idx2(h[0], p[0]), orc_idx2(h[1], p[1]));
    e -= eriv(ds, part, B, part, B, orc_idx2(h[0], p[1]), orc_idx2(h[1], p[0]));
    e *= ph;
  } else if (streq(ds, dib, djb)) {
    int h[4], p[4];
    orc_get_holes(dia, dja, nw, h);
    orc_get_parts(dia, dja, nw, p);
    double ph = orc_get_phase(dia, dja, nw, h, p, 2);
    e += eriv(ds, part, A, part, A, orc_idx2(h[0], p[0]), orc_idx2(h[1], p[1]));
    e -= eriv(ds, part, A, part, A, orc_idx2(h[0], p[1]), orc_idx2(h[1], p[0]));
    e *= ph;
  } else {
    int ha[4], pa[4], hb[4], pb[4];
    orc_get_holes(dia, dja, nw, ha);
    orc_get_parts(dia, dja, nw, pa);
    orc_get_holes(dib, djb, nw, hb);
    orc_get_parts(dib, djb, nw, pb);
    double ph = orc_get_phase(dia, dja, nw, ha, pa, 1) * orc_get_phase(dib, djb, nw, hb, pb, 1);
    e += eriv(ds, part, A, part, B, orc_idx2(ha[0], pa[0]), orc_idx2(hb[0], pb[0]));
    e *= ph;
  }
  return e;
}

/* slater_condon_mixedparticle.cpp:4-52; species ordered so a < b */
double orc_mixed_part_ham_diag(const orc_detset *ds, int a, int b, const int32_t *I, const int32_t *J) {
  (void)J;
  if (b < a) {
    int t = a;
    a = b;
    b = t;
  }
  int aA = 0, aB = beta_idx(ds, a), bA = 0, bB = beta_idx(ds, b);
  int nw = ds->n_words;
  int ao[512], av[512], bo[512], bv[512], nao, nav, nbo, nbv;
  int oao[512], oav[512], obo[512], obv[512], noao, noav, nobo, nobv;
  orc_get_occ_virt(getdet(ds, b, 0, I[b * 2 + 0]), nw, ds->d.n_orb[b], oao, &noao, oav, &noav);
  orc_get_occ_virt(getdet(ds, b, 1, I[b * 2 + 1]), nw, ds->d.n_orb[b], obo, &nobo, obv, &nobv);
  orc_get_occ_virt(getdet(ds, a, 0, I[a * 2 + 0]), nw, ds->d.n_orb[a], ao, &nao, av, &nav);
  orc_get_occ_virt(getdet(ds, a, 1, I[a * 2 + 1]), nw, ds->d.n_orb[a], bo, &nbo, bv, &nbv);
  double e = 0.0;
  for (int x = 0; x < nao; x++) {
    int i = ao[x];
    for (int y = 0; y < noao; y++) e += eriv(ds, a, aA, b, bA, orc_idx2(i, i), orc_idx2(oao[y], oao[y]));
    for (int y = 0; y < nobo; y++) e += eriv(ds, a, aA, b, bB, orc_idx2(i, i), orc_idx2(obo[y], obo[y]));
  }
  for (int x = 0; x < nbo; x++) {
    int i = bo[x];
    for (int y = 0; y < noao; y++) e += eriv(ds, a, aB, b, bA, orc_idx2(i, i), orc_idx2(oao[y], oao[y]));
    for (int y = 0; y < nobo; y++) e += eriv(ds, a, aB, b, bB, orc_idx2(i, i), orc_idx2(obo[y], obo[y]));
  }
  return e;
}

/* slater_condon_mixedparticle.cpp:54-145 */
double orc_mixed_part_ham_single(const orc_detset *ds, int a, int b, const int32_t *I, const int32_t *J) {
  if (b < a) {
    int t = a;
    a = b;
    b = t;
  }
  int nw = ds->n_words;
  const uint64_t *a_ia = getdet(ds, a, 0, I[a * 2 + 0]), *a_ib = getdet(ds, a, 1, I[a * 2 + 1]);
  const uint64_t *a_ja = getdet(ds, a, 0, J[a * 2 + 0]), *a_jb = getdet(ds, a, 1, J[a * 2 + 1]);
  const uint64_t *b_ia = getdet(ds, b, 0, I[b * 2 + 0]), *b_ib = getdet(ds, b, 1, I[b * 2 + 1]);
  const uint64_t *b_ja = getdet(ds, b, 0, J[b * 2 + 0]), *b_jb = getdet(ds, b, 1, J[b * 2 + 1]);
  int aA = 0, aB = beta_idx(ds, a), bA = 0, bB = beta_idx(ds, b);
  int ao[512], av[512], bo[512], bv[512], nao, nav, nbo, nbv;
  int h[4], p[4];
  double e = 0.0;
  if (streq(ds, b_ia, b_ja) && streq(ds, b_ib, b_jb)) {
    orc_get_occ_virt(b_ia, nw, ds->d.n_orb[b], ao, &nao, av, &nav);
    orc_get_occ_virt(b_ib, nw, ds->d.n_orb[b], bo, &nbo, bv, &nbv);
    double ph;
    int sa;
    if (streq(ds, a_ia, a_ja)) {
      orc_get_holes(a_ib, a_jb, nw, h);
      orc_get_parts(a_ib, a_jb, nw, p);
      ph = orc_get_phase(a_ib, a_jb, nw, h, p, 1);
      sa = aB;
    } else {
      orc_get_holes(a_ia, a_ja, nw, h);
      orc_get_parts(a_ia, a_ja, nw, p);
      ph = orc_get_phase(a_ia, a_ja, nw, h, p, 1);
      sa = aA;
    }
    for (int x = 0; x < nao; x++) e += eriv(ds, a, sa, b, bA, orc_idx2(h[0], p[0]), orc_idx2(ao[x], ao[x]));
    for (int x = 0; x < nbo; x++) e += eriv(ds, a, sa, b, bB, orc_idx2(h[0], p[0]), orc_idx2(bo[x], bo[x]));
    e *= ph;
  } else {
    orc_get_occ_virt(a_ia, nw, ds->d.n_orb[a], ao, &nao, av, &nav);
    orc_get_occ_virt(a_ib, nw, ds->d.n_orb[a], bo, &nbo, bv, &nbv);
    double ph;
    int sb;
    if (streq(ds, b_ib, b_jb)) {
      orc_get_holes(b_ia, b_ja, nw, h);
      orc_get_parts(b_ia, b_ja, nw, p);
      ph = orc_get_phase(b_ia, b_ja, nw, h, p, 1);
      sb = bA;
    } else {
      orc_get_holes(b_ib, b_jb, nw, h);
      orc_get_parts(b_ib, b_jb, nw, p);
      ph = orc_get_phase(b_ib, b_jb, nw, h, p, 1);
      sb = bB;
    }
    for (int x = 0; x < nao; x++) e += eriv(ds, a, aA, b, sb, orc_idx2(ao[x], ao[x]), orc_idx2(h[0], p[0]));
    for (int x = 0; x < nbo; x++) e += eriv(ds, a, aB, b, sb, orc_idx2(bo[x], bo[x]), orc_idx2(h[0], p[0]));
    e *= ph;
  }
  return e;
}

/* slater_condon_mixedparticle.cpp:147-236 */
double orc_mixed_part_ham_double(const orc_detset *ds, int a, int b, const int32_t *I, const int32_t *J) {
  if (b < a) {
    int t = a;
    a = b;
    b = t;
  }
  int nw = ds->n_words;
  const uint64_t *a_ia = getdet(ds, a, 0, I[a * 2 + 0]), *a_ib = getdet(ds, a, 1, I[a * 2 + 1]);
  const uint64_t *a_ja = getdet(ds, a, 0, J[a * 2 + 0]), *a_jb = getdet(ds, a, 1, J[a * 2 + 1]);
  const uint64_t *b_ia = getdet(ds, b, 0, I[b * 2 + 0]), *b_ib = getdet(ds, b, 1, I[b * 2 + 1]);
  const uint64_t *b_ja = getdet(ds, b, 0, J[b * 2 + 0]), *b_jb = getdet(ds, b, 1, J[b * 2 + 1]);
  int aA = 0, aB = beta_idx(ds, a), bA = 0, bB = beta_idx(ds, b);
  const uint64_t *ai, *aj, *bi, *bj;
  int sa, sb;
  if (streq(ds, a_ia, a_ja) && streq(ds, b_ia, b_ja)) {
    ai = a_ib, aj = a_jb, bi = b_ib, bj = b_jb, sa = aB, sb = bB;
  } else if (streq(ds, a_ib, a_jb) && streq(ds, b_ib, b_jb)) {
    ai = a_ia, aj = a_ja, bi = b_ia, bj = b_ja, sa = aA, sb = bA;
  } else if (streq(ds, a_ia, a_ja) && streq(ds, b_ib, b_jb)) {
    ai = a_ib, aj = a_jb, bi = b_ia, bj = b_ja, sa = aB, sb = bA;
  } else if (streq(ds, a_ib, a_jb) && streq(ds, b_ia, b_ja)) {
    ai = a_ia, aj = a_ja, bi = b_ib, bj = b_jb, sa = aA, sb = bB;
  } else {
    return 0.0;
  }
  int ha[4], pa[4], hb[4], pb[4];
  orc_get_holes(ai, aj, nw, ha);
  orc_get_parts(ai, aj, nw, pa);
  orc_get_holes(bi, bj, nw, hb);
  orc_get_parts(bi, bj, nw, pb);
  double ph = orc_get_phase(ai, aj, nw, ha, pa, 1) * orc_get_phase(bi, bj, nw, hb, pb, 1);
  return ph * eriv(ds, a, sa, b, sb, orc_idx2(ha[0], pa[0]), orc_idx2(hb[0], pb[0]));
}

static inline int num_exc_part(const orc_detset *ds, int part, const int32_t *I, const int32_t *J) {
  return orc_single_spin_num_excitation(getdet(ds, part, 0, I[part * 2]), getdet(ds, part, 0, J[part * 2]), ds->n_words) +
         orc_single_spin_num_excitation(getdet(ds, part, 1, I[part * 2 + 1]), getdet(ds, part, 1, J[part * 2 + 1]), ds->n_words);
}

/* slater_condon.cpp:102-153; the mixed diagonal term is added once */
const double *orc_diagonal(orc_detset *ds) {
  if (ds->diag) return ds->diag;
  int64_t nd = ds->n_dets;
  ds->diag = (double *)calloc((size_t)(nd > 0 ? nd : 1), sizeof(double));
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < nd; i++) {
    const int32_t *u = ds->unfold + i * ds->ntup;
    double e = 0.0;
    for (int p = 0; p < ds->d.n_species; p++) e += orc_same_part_ham_diag(ds, p, u, u);
    if (ds->d.n_species == 2) e += ds->d.charge[0] * ds->d.charge[1] * orc_mixed_part_ham_diag(ds, 1, 0, u, u);
    ds->diag[i] = e;
  }
  return ds->diag;
}

/* slater_condon.cpp:4-100.  For two species the loop over "other" species only
 * reaches the pair (1, 0) (the `continue` skips the increment), so the cross
 * term is added exactly once. */
double orc_slater_condon(orc_detset *ds, int64_t i, int64_t j) {
  if (i == j) return orc_diagonal(ds)[i];
  const int32_t *I = ds->unfold + i * ds->ntup, *J = ds->unfold + j * ds->ntup;
  int ns = ds->d.n_species;
  int eq[2];
  for (int p = 0; p < ns; p++) eq[p] = (I[2 * p] == J[2 * p]) && (I[2 * p + 1] == J[2 * p + 1]);
  double e = 0.0;
  for (int p = 0; p < ns; p++) {
    int others_equal = 1;
    for (int q = 0; q < ns; q++)
      if (q != p && !eq[q]) others_equal = 0;
    if (others_equal) {
      int ex = num_exc_part(ds, p, I, J);
      if (ex == 0)
        e += orc_same_part_ham_diag(ds, p, I, J);
      else if (ex == 1)
        e += orc_same_part_ham_single(ds, p, I, J);
      else if (ex == 2)
        e += orc_same_part_ham_double(ds, p, I, J);
    }
  }
  if (ns == 2) {
    int exi = num_exc_part(ds, 1, I, J), exj = num_exc_part(ds, 0, I, J);
    double cf = ds->d.charge[0] * ds->d.charge[1];
    if (exi + exj < 3) {
      if (exi == 0 && exj == 0)
        e += cf * orc_mixed_part_ham_diag(ds, 1, 0, I, J);
      else if (exi == 1 && exj == 1)
        e += cf * orc_mixed_part_ham_double(ds, 1, 0, I, J);
      else if (exi == 1 || exj == 1)
        e += cf * orc_mixed_part_ham_single(ds, 1, 0, I, J);
    }
  }
  return e;
}

/* ------------------------------------------------------------------------- */
/* pair-once accumulation used by the singleshot restatements */
static inline void pair_update(double *S, int64_t lds, const double *C, int64_t ldc, int nvec, int64_t i, int64_t j, double h) {
  if (h == 0.0) return;
  for (int v = 0; v < nvec; v++) {
    S[i + v * lds] += h * C[j + v * ldc];
    S[j + v * lds] += h * C[i + v * ldc];
  }
}

static int get_threads(int nthreads) {
#ifdef _OPENMP
  return nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
  return 1;
#endif
}

/* direct_singleparticle.cpp:238-372 (sigma_one_species_class_singleshot) */
static void sigma_one_species(orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
  const double *diag = orc_diagonal(ds);
  int64_t nd = ds->n_dets;
  int nt = get_threads(nthreads);
  double **priv = (double **)calloc((size_t)nt, sizeof(double *));
  for (int t = 0; t < nt; t++) priv[t] = (double *)calloc((size_t)nd * nvec, sizeof(double));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
    int nth = omp_get_num_threads();
#else
    int tid = 0, nth = 1;
#endif
    double *P = priv[tid];
    for (int64_t i = 0; i < nd; i++) {
      if (i % nth != tid) continue;
      const int32_t *I = ds->unfold + i * 2;
      int32_t IA = I[0], IB = I[1];
      for (int v = 0; v < nvec; v++) P[i + v * nd] += diag[i] * C[i + v * ldc];
      const int32_t *sa, *sb, *da, *db;
      int64_t nsa = orc_singles(ds, 0, 0, IA, &sa), nsb = orc_singles(ds, 0, 1, IB, &sb);
      int64_t nda = orc_doubles(ds, 0, 0, IA, &da), ndb = orc_doubles(ds, 0, 1, IB, &db);
      for (int64_t x = 0; x < nsa; x++) {
        int32_t JA = sa[x];
        if (JA < IA) continue;
        int32_t J[2] = {JA, IB};
        int64_t j = orc_lookup(ds, J);
        if (j >= 0) pair_update(P, nd, C, ldc, nvec, i, j, orc_same_part_ham_single(ds, 0, I, J));
        for (int64_t y = 0; y < nsb; y++) {
          int32_t J2[2] = {JA, sb[y]};
          int64_t j2 = orc_lookup(ds, J2);
          if (j2 >= 0) pair_update(P, nd, C, ldc, nvec, i, j2, orc_same_part_ham_double(ds, 0, I, J2));
        }
      }
      for (int64_t y = 0; y < nsb; y++) {
        int32_t JB = sb[y];
        if (JB < IB) continue;
        int32_t J[2] = {IA, JB};
        int64_t j = orc_lookup(ds, J);
        if (j >= 0) pair_update(P, nd, C, ldc, nvec, i, j, orc_same_part_ham_single(ds, 0, I, J));
      }
      for (int64_t x = 0; x < nda; x++) {
        int32_t JA = da[x];
        if (JA < IA) continue;
        int32_t J[2] = {JA, IB};
        int64_t j = orc_lookup(ds, J);
        if (j >= 0) pair_update(P, nd, C, ldc, nvec, i, j, orc_same_part_ham_double(ds, 0, I, J));
      }
      for (int64_t y = 0; y < ndb; y++) {
        int32_t JB = db[y];
        if (JB < IB) continue;
        int32_t J[2] = {IA, JB};
        int64_t j = orc_lookup(ds, J);
        if (j >= 0) pair_update(P, nd, C, ldc, nvec, i, j, orc_same_part_ham_double(ds, 0, I, J));
      }
    }
#pragma omp critical
    {
      for (int v = 0; v < nvec; v++)
        for (int64_t i = 0; i < nd; i++) S[i + v * lds] += P[i + v * nd];
    }
  }
  for (int t = 0; t < nt; t++) free(priv[t]);
  free(priv);
}

/* direct_mixedparticle.cpp:269-611 (sigma_two_species_class_singleshot) */
static void sigma_two_species(orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
  const double *diag = orc_diagonal(ds);
  int64_t nd = ds->n_dets;
  double cf = ds->d.charge[0] * ds->d.charge[1];
  int nt = get_threads(nthreads);
  double **priv = (double **)calloc((size_t)nt, sizeof(double *));
  for (int t = 0; t < nt; t++) priv[t] = (double *)calloc((size_t)nd * nvec, sizeof(double));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    int tid = omp_get_thread_num();
    int nth = omp_get_num_threads();
#else
    int tid = 0, nth = 1;
#endif
    double *P = priv[tid];
    for (int64_t i = 0; i < nd; i++) {
      if (i % nth != tid) continue;
      const int32_t *I = ds->unfold + i * 4;
      for (int v = 0; v < nvec; v++) P[i + v * nd] += diag[i] * C[i + v * ldc];
      const int32_t *s1[4], *s2[4];
      int64_t n1[4], n2[4];
      for (int q = 0; q < 4; q++) {
        n1[q] = orc_singles(ds, q / 2, q % 2, I[q], &s1[q]);
        n2[q] = orc_doubles(ds, q / 2, q % 2, I[q], &s2[q]);
      }
      /* singles in slot q (alpha/beta of species 0/1), each followed by the
       * single x single doubles with every later slot (:305-517) */
      for (int q = 0; q < 4; q++) {
        for (int64_t x = 0; x < n1[q]; x++) {
          int32_t Jq = s1[q][x];
          if (Jq < I[q]) continue;
          int32_t J[4] = {I[0], I[1], I[2], I[3]};
          J[q] = Jq;
          int64_t j = orc_lookup(ds, J);
          if (j >= 0) {
            double h = orc_same_part_ham_single(ds, q / 2, I, J) + cf * orc_mixed_part_ham_single(ds, 0, 1, I, J);
            pair_update(P, nd, C, ldc, nvec, i, j, h);
          }
          for (int r = q + 1; r < 4; r++) {
            for (int64_t y = 0; y < n1[r]; y++) {
              int32_t J2[4] = {J[0], J[1], J[2], J[3]};
              J2[r] = s1[r][y];
              int64_t j2 = orc_lookup(ds, J2);
              if (j2 < 0) continue;
              double h2;
              if (q == 0 && r == 1)
                h2 = orc_same_part_ham_double(ds, 0, I, J2) + cf * orc_mixed_part_ham_double(ds, 0, 1, I, J2);
              else if (q == 2 && r == 3)
                h2 = orc_same_part_ham_double(ds, 1, I, J2) + cf * orc_mixed_part_ham_double(ds, 0, 1, I, J2);
              else
                h2 = cf * orc_mixed_part_ham_double(ds, 0, 1, I, J2);
              pair_update(P, nd, C, ldc, nvec, i, j2, h2);
            }
          }
        }
      }
      /* same-spin doubles (:519-605) */
      for (int q = 0; q < 4; q++) {
        for (int64_t x = 0; x < n2[q]; x++) {
          int32_t Jq = s2[q][x];
          if (Jq < I[q]) continue;
          int32_t J[4] = {I[0], I[1], I[2], I[3]};
          J[q] = Jq;
          int64_t j = orc_lookup(ds, J);
          if (j >= 0) pair_update(P, nd, C, ldc, nvec, i, j, orc_same_part_ham_double(ds, q / 2, I, J));
        }
      }
    }
#pragma omp critical
    {
      for (int v = 0; v < nvec; v++)
        for (int64_t i = 0; i < nd; i++) S[i + v * lds] += P[i + v * nd];
    }
  }
  for (int t = 0; t < nt; t++) free(priv[t]);
  free(priv);
}

/* direct.cpp:21-33 (create_sigma); S is overwritten */
void orc_sigma_singleshot(orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
  for (int v = 0; v < nvec; v++) memset(S + v * lds, 0, sizeof(double) * (size_t)ds->n_dets);
  if (ds->d.n_species == 1)
    sigma_one_species(ds, C, ldc, nvec, S, lds, nthreads);
  else
    sigma_two_species(ds, C, ldc, nvec, S, lds, nthreads);
}

/* direct.cpp:36-52 (create_sigma_slow): dense product through Slater_Condon */
void orc_sigma_slow(orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads) {
  orc_diagonal(ds);
  int64_t nd = ds->n_dets;
  int nt = get_threads(nthreads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
  for (int64_t i = 0; i < nd; i++) {
    for (int v = 0; v < nvec; v++) S[i + v * lds] = 0.0;
    for (int64_t k = 0; k < nd; k++) {
      double h = orc_slater_condon(ds, i, k);
      if (h != 0.0)
        for (int v = 0; v < nvec; v++) S[i + v * lds] += h * C[k + v * ldc];
    }
  }
}

void orc_dense_ham(orc_detset *ds, double *H, int nthreads) {
  orc_diagonal(ds);
  int64_t nd = ds->n_dets;
  int nt = get_threads(nthreads);
#pragma omp parallel for num_threads(nt) schedule(dynamic, 4)
  for (int64_t j = 0; j < nd; j++)
    for (int64_t i = 0; i < nd; i++) H[i + j * nd] = orc_slater_condon(ds, i, j);
}

/* Gather form of the same operator: for each listed row I, sum H_IJ C_J over
 * every connected J (both directions of each pair), using the same element
 * formulas as the singleshot builders. */
void orc_sigma_rows(orc_detset *ds, const double *C, int64_t ldc, int nvec, const int64_t *rows, int64_t n_rows, double *S_rows,
                    int nthreads) {
  const double *diag = orc_diagonal(ds);
  int ns = ds->d.n_species;
  double cf = ns == 2 ? ds->d.charge[0] * ds->d.charge[1] : 0.0;
  int nt = get_threads(nthreads);
  int nslot = 2 * ns;
#pragma omp parallel for num_threads(nt) schedule(dynamic, 1)
  for (int64_t r = 0; r < n_rows; r++) {
    int64_t i = rows[r];
    const int32_t *I = ds->unfold + i * ds->ntup;
    double acc[64];
    for (int v = 0; v < nvec; v++) acc[v] = diag[i] * C[i + v * ldc];
    const int32_t *s1[4], *s2[4];
    int64_t n1[4], n2[4];
    for (int q = 0; q < nslot; q++) {
      n1[q] = orc_singles(ds, q / 2, q % 2, I[q], &s1[q]);
      n2[q] = orc_doubles(ds, q / 2, q % 2, I[q], &s2[q]);
    }
    for (int q = 0; q < nslot; q++) {
      for (int64_t x = 0; x < n1[q]; x++) {
        int32_t J[4] = {I[0], I[1], ns == 2 ? I[2] : 0, ns == 2 ? I[3] : 0};
        J[q] = s1[q][x];
        int64_t j = orc_lookup(ds, J);
        if (j >= 0) {
          double h = orc_same_part_ham_single(ds, q / 2, I, J);
          if (ns == 2) h += cf * orc_mixed_part_ham_single(ds, 0, 1, I, J);
          if (h != 0.0)
            for (int v = 0; v < nvec; v++) acc[v] += h * C[j + v * ldc];
        }
        for (int r2 = q + 1; r2 < nslot; r2++) {
          for (int64_t y = 0; y < n1[r2]; y++) {
            int32_t J2[4] = {J[0], J[1], J[2], J[3]};
            J2[r2] = s1[r2][y];
            int64_t j2 = orc_lookup(ds, J2);
            if (j2 < 0) continue;
            double h2;
            if (q == 0 && r2 == 1) {
              h2 = orc_same_part_ham_double(ds, 0, I, J2);
              if (ns == 2) h2 += cf * orc_mixed_part_ham_double(ds, 0, 1, I, J2);
            } else if (q == 2 && r2 == 3) {
              h2 = orc_same_part_ham_double(ds, 1, I, J2) + cf * orc_mixed_part_ham_double(ds, 0, 1, I, J2);
            } else {
              h2 = cf * orc_mixed_part_ham_double(ds, 0, 1, I, J2);
            }
            if (h2 != 0.0)
              for (int v = 0; v < nvec; v++) acc[v] += h2 * C[j2 + v * ldc];
          }
        }
      }
      for (int64_t x = 0; x < n2[q]; x++) {
        int32_t J[4] = {I[0], I[1], ns == 2 ? I[2] : 0, ns == 2 ? I[3] : 0};
        J[q] = s2[q][x];
        int64_t j = orc_lookup(ds, J);
        if (j >= 0) {
          double h = orc_same_part_ham_double(ds, q / 2, I, J);
          if (h != 0.0)
            for (int v = 0; v < nvec; v++) acc[v] += h * C[j + v * ldc];
        }
      }
    }
    for (int v = 0; v < nvec; v++) S_rows[r + v * n_rows] = acc[v];
  }
}

/* ------------------------------------------------------------------------- */
/* s2.cpp:4-123 (evaluate_s2).  Per determinant and species: the diagonal
 * n_a + s_z (s_z - 1) over the open shells, then every alpha single x beta
 * single partner whose hole of one spin is the particle of the other
 * subtracts phase_a * phase_b * C_I * C_J.  S2 is nvec x n_species,
 * column-major. */
void orc_evaluate_s2(const orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S2, int nthreads) {
  const int nsp = ds->d.n_species, nw = ds->n_words, ntup = ds->ntup;
  const int nt = get_threads(nthreads);
  double *part = (double *)calloc((size_t)nt * nvec * nsp, sizeof(double));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    double *acc = part + (size_t)omp_get_thread_num() * nvec * nsp;
#else
    double *acc = part;
#endif
    int ha[64 * MAXW], pa[64 * MAXW], hb[64 * MAXW], pb[64 * MAXW];
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < ds->n_dets; i++) {
      const int32_t *iu = ds->unfold + i * ntup;
      for (int v = 0; v < nvec; v++) {
        const double ci = C[i + v * ldc];
        if (ci == 0.0) continue;
        for (int p = 0; p < nsp; p++) {
          const int32_t ia = iu[2 * p], ib = iu[2 * p + 1];
          const uint64_t *Da = getdet(ds, p, 0, ia), *Db = getdet(ds, p, 1, ib);
          int n_tot = 0, n_a = 0;
          for (int w = 0; w < nw; w++) {
            const uint64_t x = Da[w] ^ Db[w];
            n_tot += __builtin_popcountll(x);
            n_a += __builtin_popcountll(x & Da[w]);
          }
          const double sz = n_a - 0.5 * n_tot;
          acc[v + p * nvec] += ci * ci * (n_a + sz * (sz - 1.0));
          const int32_t *la, *lb;
          const int64_t na = orc_singles(ds, p, 0, ia, &la), nb = orc_singles(ds, p, 1, ib, &lb);
          for (int64_t x = 0; x < na; x++)
            for (int64_t y = 0; y < nb; y++) {
              int32_t t[4] = {iu[0], iu[1], ntup > 2 ? iu[2] : 0, ntup > 2 ? iu[3] : 0};
              t[2 * p] = la[x];
              t[2 * p + 1] = lb[y];
              const int64_t j = orc_lookup(ds, t);
              if (j < 0) continue;
              const double cj = C[j + v * ldc];
              if (cj == 0.0) continue;
              const uint64_t *Ja = getdet(ds, p, 0, la[x]), *Jb = getdet(ds, p, 1, lb[y]);
              orc_get_holes(Da, Ja, nw, ha);
              orc_get_parts(Da, Ja, nw, pa);
              orc_get_holes(Db, Jb, nw, hb);
              orc_get_parts(Db, Jb, nw, pb);
              if (ha[0] == pb[0] && hb[0] == pa[0]) {
                const double ph = orc_get_phase(Da, Ja, nw, ha, pa, 1) * orc_get_phase(Db, Jb, nw, hb, pb, 1);
                acc[v + p * nvec] -= ph * ci * cj;
              }
            }
        }
      }
    }
  }
  for (int k = 0; k < nvec * nsp; k++) {
    double s = 0.0;
    for (int t = 0; t < nt; t++) s += part[(size_t)t * nvec * nsp + k];
    S2[k] = s;
  }
  free(part);
}

/* rdm1.cpp:4-72 (create_1rdm) for one species and spin: C_I^2 on the diagonal
 * of each occupied orbital, and for each single partner J < I the product
 * phase C_I C_J added at (hole, particle) and (particle, hole); contributions
 * with magnitude <= 1e-16 are skipped.  All orbitals are taken as one irrep
 * (the reference's symmetry-label filter admits every pair without point-group
 * symmetry).  rdm is n_orb x n_orb, column-major. */
void orc_create_1rdm(const orc_detset *ds, const double *c, int part, int spin, double *rdm, int nthreads) {
  const int n = ds->d.n_orb[part], nw = ds->n_words, ntup = ds->ntup, slot = 2 * part + spin;
  const double thresh = 1e-16;
  const int nt = get_threads(nthreads);
  double *acc_all = (double *)calloc((size_t)nt * n * n, sizeof(double));
#pragma omp parallel num_threads(nt)
  {
#ifdef _OPENMP
    double *acc = acc_all + (size_t)omp_get_thread_num() * n * n;
#else
    double *acc = acc_all;
#endif
    int occ[64 * MAXW], virt[64 * MAXW], h[64 * MAXW], q[64 * MAXW];
#pragma omp for schedule(dynamic, 16)
    for (int64_t i = 0; i < ds->n_dets; i++) {
      const int32_t *iu = ds->unfold + i * ntup;
      const int32_t si = iu[slot];
      const uint64_t *Di = getdet(ds, part, spin, si);
      int no = 0, nv = 0;
      orc_get_occ_virt(Di, nw, n, occ, &no, virt, &nv);
      const double d = c[i] * c[i];
      if (fabs(d) > thresh)
        for (int k = 0; k < no; k++) acc[occ[k] + (int64_t)occ[k] * n] += d;
      const int32_t *ls;
      const int64_t ns = orc_singles(ds, part, spin, si, &ls);
      for (int64_t x = 0; x < ns; x++) {
        int32_t t[4] = {iu[0], iu[1], ntup > 2 ? iu[2] : 0, ntup > 2 ? iu[3] : 0};
        t[slot] = ls[x];
        const int64_t j = orc_lookup(ds, t);
        if (j < 0 || i < j) continue;
        const uint64_t *Dj = getdet(ds, part, spin, ls[x]);
        orc_get_holes(Di, Dj, nw, h);
        orc_get_parts(Di, Dj, nw, q);
        const double v = orc_get_phase(Di, Dj, nw, h, q, 1) * c[i] * c[j];
        if (fabs(v) > thresh) {
          acc[h[0] + (int64_t)q[0] * n] += v;
          acc[q[0] + (int64_t)h[0] * n] += v;
        }
      }
    }
  }
  for (int64_t k = 0; k < (int64_t)n * n; k++) {
    double s = 0.0;
    for (int t = 0; t < nt; t++) s += acc_all[(size_t)t * n * n + k];
    rdm[k] = s;
  }
  free(acc_all);
}
