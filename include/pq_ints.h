/*
 * pq_ints.h -- C ABI of the GB300 AO->MO two-electron integral transform.
 *
 * Replaces POLYQUANT_INTEGRAL::transform_mo_2_body_integrals
 * (src/integral/integral.hpp:201-204, src/integral/integral.cpp:207-477) for
 * one (species a, spin a, species b, spin b) block, as called by
 * calculate_mo_2_body_integrals (integral.cpp:479-516).  The reference forms
 * the AO integrals shell-quartet by shell-quartet inside the first quarter
 * transform; here the AO integrals are an input already resident on the device.
 *
 * Output layout is the reference's: an (npair_mo_a x npair_mo_b) column-major
 * matrix, element [idx2(i,j) + idx2(k,l) * npair_mo_a] = (ij|kl) with
 * idx2(i,j) = max(i,j)(max(i,j)+1)/2 + min(i,j) (integral.hpp:14-20).
 * Frozen-core / deleted-virtual offsets are applied by the caller by passing
 * C already offset to the first active column with ldc = n_ao.
 */
#ifndef PQ_INTS_H
#define PQ_INTS_H
#include <stdint.h>

#include "pq_ci.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
  PQ_AO_PACKED8 = 0, /* same species: idx2(idx2(mu,nu), idx2(la,si)) packed, npair(npair+1)/2 values */
  PQ_AO_PAIRS = 1    /* any two species: (npair_a x npair_b) column-major pair matrix */
};

enum {
  PQ_XFORM_FP64 = 0,   /* plain FP64 quarter transforms */
  PQ_XFORM_BF16X3 = 1, /* split-BF16 (hi*hi + hi*lo + lo*hi) on tcgen05, FP32 accumulate */
  PQ_XFORM_TF32X3 = 2  /* split-TF32 (hi*hi + hi*lo + lo*hi) on tcgen05, FP32 accumulate */
};

/* All pointers are DEVICE buffers.  C_a: n_ao_a x n_mo_a column-major with
 * leading dimension ldc_a (>= n_ao_a); likewise C_b.  stream: cudaStream_t or
 * NULL.  For PQ_AO_PACKED8 the two species must be the same (n_ao_a == n_ao_b). */
pq_status pq_ao2mo(const double *eri_ao, int32_t layout, int64_t n_ao_a, int64_t n_ao_b, const double *C_a,
                   int64_t ldc_a, int64_t n_mo_a, const double *C_b, int64_t ldc_b, int64_t n_mo_b, int32_t mode,
                   double *eri_mo, void *stream);

/* The split-precision modes keep their work buffers (about 2.5 x the FP64
 * pair matrix, e.g. 20 GB at n_ao = n_mo = 256) on the device between calls,
 * so repeated transforms allocate nothing; calls on one device share them and
 * run one at a time.  This frees them for the current device (no reference
 * counterpart: the reference's transform holds its buffers only during the
 * call). */
pq_status pq_ao2mo_release_workspace(void);

/* MO one-body integrals h_MO = C^T F C for an n_ao x n_ao operator F
 * (integral.cpp:166-205); DEVICE buffers, column-major. */
pq_status pq_mo1(const double *F_ao, int64_t n_ao, const double *C, int64_t ldc, int64_t n_mo, double *h_mo,
                 void *stream);

/* Diagnostic hook, no reference counterpart: budget, in SM clock cycles, of
 * the waits inside the tensor-core GEMM pipeline (<= 0 restores the default of
 * about 2 s).  A wait that runs out makes the transform return PQ_TIMEOUT
 * after the kernel has waited (with the default budget) for its own loads and
 * MMAs and freed its tensor memory; the context stays usable.  Meant for
 * tests of that path. */
pq_status pq_debug_set_wait_budget(long long cycles);

#ifdef __cplusplus
}
#endif
#endif
