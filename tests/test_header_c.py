"""The public headers are plain C: a C99 translation unit that calls every entry point compiles and links
against the library (no GPU needed; nothing is executed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <stddef.h>
#include "pq_ci.h"
#include "pq_ints.h"

int use_all(void) {
  pq_ci_desc d = {0};
  pq_ci_handle *h = 0;
  pq_ci_batch *b = 0;
  pq_davidson_params p = {0};
  pq_davidson_report r = {0};
  int64_t n = 0, nnz = 0;
  int32_t nw = 0, w = 0, rows = 0;
  double e[4], s2[4];
  const char *msg = pq_last_error();
  const char *ver = pq_version();
  (void)msg; (void)ver;
  pq_status st = pq_ci_create(&d, NULL, &h);
  st |= pq_ci_num_dets(h, &n);
  st |= pq_ci_strings(h, 0, 0, NULL, &n, &nw);
  st |= pq_ci_det_unfold(h, NULL);
  st |= pq_ci_diag(h, NULL);
  st |= pq_ci_sigma(h, NULL, n, 1, NULL, n, PQ_FP64);
  st |= pq_ci_sigma_host(h, NULL, n, 1, NULL, n, PQ_FP32);
  st |= pq_ci_sigma_noalloc(h, NULL, n, 1, NULL, n, PQ_FP64);
  st |= pq_ci_sigma_interleaved(h, NULL, NULL, 4, PQ_FP32, 0.0);
  st |= pq_ci_davidson(h, &p, e, NULL, &r);
  st |= pq_ci_ham_build(h, 0.0, 1, &nnz);
  st |= pq_ci_ham_csr(h, 1, &nnz, NULL, NULL, NULL);
  st |= pq_ci_ham_release(h);
  st |= pq_ci_s2(h, NULL, n, 1, s2);
  st |= pq_ci_rdm1(h, NULL, 0, 0, NULL);
  {
    double v = 0.0;
    int64_t I = 0, J = 0, bytes = 0;
    st |= pq_ci_element(h, 0, 0, &v);
    st |= pq_ci_elements(h, 1, &I, &J, &v);
    st |= pq_debug_scratch_bytes(h, &bytes);
  }
  st |= pq_ci_destroy(h);
  {
    const uint64_t hf = 3;
    const uint64_t *lists[2] = {&hf, &hf};
    const int64_t counts[2] = {1, 1};
    st |= pq_ci_create_selected(&d, lists, counts, NULL, &h);
  }
  st |= pq_ci_batch_create(&d, 1, NULL, &b);
  st |= pq_ci_batch_num_dets(b, 0, &n);
  st |= pq_ci_batch_sigma(b, NULL, NULL, 1, NULL, NULL, PQ_FP64);
  st |= pq_ci_batch_tuning(b, &w, &rows);
  st |= pq_ci_batch_davidson(b, &p, 0, e, &r);
  st |= pq_ci_batch_destroy(b);
  st |= pq_ao2mo(NULL, PQ_AO_PACKED8, 1, 1, NULL, 1, 1, NULL, 1, 1, PQ_XFORM_BF16X3, NULL, NULL);
  st |= pq_mo1(NULL, 1, NULL, 1, 1, NULL, NULL);
  st |= pq_ao2mo_release_workspace();
  st |= pq_debug_set_wait_budget(0);
  return (int)st;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_headers_compile_as_c99_and_link(tmp_path):
    lib = os.path.join(ROOT, "polyquant_gb300", "lib")
    if not os.path.exists(os.path.join(lib, "libpq_gb300.so")):
        pytest.skip("library not built")
    src = tmp_path / "use_all.c"
    src.write_text(SRC + "\nint main(void) { return 0; }\n")
    exe = tmp_path / "use_all"
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                        str(exe), "-L", lib, "-lpq_gb300", "-Wl,-rpath," + lib, "-Wl,--unresolved-symbols=ignore-in-shared-libs"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
