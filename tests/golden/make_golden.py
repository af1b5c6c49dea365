"""Regenerate tests/golden/h2o_sto3g_golden.npz from the reference's own fixtures.

Run once in a checkout that has the polyquant sources at $POLYQUANT_REF
(default /root/reference); the npz is committed so that the tests never read
the reference tree at run time.

Sources (paths inside the polyquant project):
  tests/data/h2o_sto3glibrary_cisd/cisd_ham_elements.txt  141x141 CISD H, column 0
      (compared in tests/integration_tests/calculation/calculation_test.cpp:253-307)
  tests/data/h2o_sto3glibrary_cisd/ref_mo_onebody.txt      5x5 h_MO, sto3galls basis
  tests/data/h2o_sto3glibrary_cisd/ref_eri.txt             (ij|kl) i<=j, k<=l, same basis
      (both compared in tests/unit_tests/ci/ci_test.cpp:12-70)
"""
import os

import numpy as np

REF = os.environ.get("POLYQUANT_REF", "/root/reference")
D = os.path.join(REF, "tests", "data", "h2o_sto3glibrary_cisd")


def main():
    ham = np.loadtxt(os.path.join(D, "cisd_ham_elements.txt"))[:, 0].reshape(141, 141)
    h1 = np.loadtxt(os.path.join(D, "ref_mo_onebody.txt"))
    eri = np.loadtxt(os.path.join(D, "ref_eri.txt"))
    out = os.path.join(os.path.dirname(os.path.abspath(__file__)), "h2o_sto3g_golden.npz")
    np.savez_compressed(out, cisd_ham=ham, alls_h1=h1, alls_eri=eri)
    print("wrote", out)


if __name__ == "__main__":
    main()
