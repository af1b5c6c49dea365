/*
 * pq_oracle.h -- CPU oracle for the polyquant CI sigma / Slater-Condon path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithms (polyquant src/ci/detset/ sources) used as the checker for the GPU
 * library and as the timed CPU baseline.  Nothing in the product library links
 * or calls it.
 */
#ifndef PQ_ORACLE_H
#define PQ_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Same field layout as pq_ci_desc in include/pq_ci.h (checked by a test). */
typedef struct {
  int32_t n_species;
  int32_t n_orb[2];
  int32_t n_alpha[2];
  int32_t n_beta[2];
  int32_t restricted[2];
  double charge[2];
  int32_t ex_level[2][3];
  int32_t max_collective;
  const double *h1[2][2];
  const double *eri[2][2][2][2];
} orc_desc;

typedef struct orc_detset orc_detset;

/* ---- bit operations on multi-word strings (determinant_operations.cpp) ---- */
int orc_single_spin_num_excitation(const uint64_t *Di, const uint64_t *Dj, int n_words);
int orc_get_holes(const uint64_t *Di, const uint64_t *Dj, int n_words, int *holes);
int orc_get_parts(const uint64_t *Di, const uint64_t *Dj, int n_words, int *parts);
double orc_get_phase(const uint64_t *Di, const uint64_t *Dj, int n_words, const int *holes, const int *parts, int n_exc);
int orc_get_occ_virt(const uint64_t *D, int n_words, int max_orb, int *occ, int *n_occ, int *virt, int *n_virt);
int orc_idx2(int i, int j);

/* ---- determinant set ---- */
orc_detset *orc_detset_create(const orc_desc *d, int check_addressing);
void orc_detset_destroy(orc_detset *ds);
int orc_n_words(const orc_detset *ds);
int64_t orc_n_dets(const orc_detset *ds);
int64_t orc_n_strings(const orc_detset *ds, int species, int spin);
const uint64_t *orc_strings(const orc_detset *ds, int species, int spin);
const int32_t *orc_unfold(const orc_detset *ds); /* n_dets x (2*n_species) */
int64_t orc_lookup(const orc_detset *ds, const int32_t *tuple);
int64_t orc_singles(const orc_detset *ds, int species, int spin, int64_t I, const int32_t **list);
int64_t orc_doubles(const orc_detset *ds, int species, int spin, int64_t I, const int32_t **list);
const double *orc_diagonal(orc_detset *ds); /* computes on first call */

/* ---- matrix elements (slater_condon*.cpp) ---- */
double orc_same_part_ham_diag(const orc_detset *ds, int part, const int32_t *I, const int32_t *J);
double orc_same_part_ham_single(const orc_detset *ds, int part, const int32_t *I, const int32_t *J);
double orc_same_part_ham_double(const orc_detset *ds, int part, const int32_t *I, const int32_t *J);
double orc_mixed_part_ham_diag(const orc_detset *ds, int a, int b, const int32_t *I, const int32_t *J);
double orc_mixed_part_ham_single(const orc_detset *ds, int a, int b, const int32_t *I, const int32_t *J);
double orc_mixed_part_ham_double(const orc_detset *ds, int a, int b, const int32_t *I, const int32_t *J);
double orc_slater_condon(orc_detset *ds, int64_t i, int64_t j);

/* ---- sigma builders (direct*.cpp); C and S are N x nvec column-major ---- */
void orc_sigma_singleshot(orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads);
void orc_sigma_slow(orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S, int64_t lds, int nthreads);
/* gather form: exact sigma rows for the listed determinants (any order) */
void orc_sigma_rows(orc_detset *ds, const double *C, int64_t ldc, int nvec, const int64_t *rows, int64_t n_rows,
                    double *S_rows /* n_rows x nvec col-major */, int nthreads);
/* explicit dense H (n_dets x n_dets, col-major), small cases only */
void orc_dense_ham(orc_detset *ds, double *H, int nthreads);

/* ---- properties of CI vectors (s2.cpp, rdm1.cpp) ---- */
/* <S^2> per vector and species: S2 is nvec x n_species, col-major */
void orc_evaluate_s2(const orc_detset *ds, const double *C, int64_t ldc, int nvec, double *S2, int nthreads);
/* one-particle density matrix of one species and spin: n_orb x n_orb, col-major */
void orc_create_1rdm(const orc_detset *ds, const double *c, int part, int spin, double *rdm, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
