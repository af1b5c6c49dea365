"""Regenerate the golden fixtures of tests/golden/ from the reference's own test data.

Run once with the environment variable POLYQUANT_REF set to the root of a
polyquant source checkout (the directory holding tests/data/); the npz files
are committed so that the tests never read the reference tree at run time.

Sources (paths inside the polyquant project):
  h2o_sto3g_golden.npz
    tests/data/h2o_sto3glibrary_cisd/cisd_ham_elements.txt  141x141 CISD H, column 0
        (compared in tests/integration_tests/calculation/calculation_test.cpp:253-307)
    tests/data/h2o_sto3glibrary_cisd/ref_mo_onebody.txt      5x5 h_MO, sto3galls basis
    tests/data/h2o_sto3glibrary_cisd/ref_eri.txt             (ij|kl) i<=j, k<=l, same basis
        (both compared in tests/unit_tests/ci/ci_test.cpp:12-70)
  h_minus_no_golden.npz
    tests/data/PsH_wpos/electron_basis.g94   the s basis of H- (five contracted shells)
    tests/data/PsH_wpos/h_minus_NO_occ.txt   natural-orbital occupations (spin-summed)
    tests/data/PsH_wpos/h_minus_NO.txt       natural orbitals in the AO basis
        (compared in tests/unit_tests/ci/ci_test.cpp:854-871, "CI: Natural Orbitals";
         input tests/data/PsH_wpos/H_minus.json: RHF, CISD [1,1,2], state 0)
  positron_bases.npz
    tests/data/li-_custombasis_wpos/Li_basis.g94   s and p shells of Li_wpos.json (electron and positron)
    tests/data/PsH_wpos/electron_basis.g94, positron_basis.g94   the bases of PsH_wpos_CI.json
"""
import os

import numpy as np

REF = os.environ.get("POLYQUANT_REF", "")
HERE = os.path.dirname(os.path.abspath(__file__))


def read_g94(path):
    """[(kind, [(exponent, coefficient), ...]), ...] of a one-element Gaussian-94 basis file (s and p shells)."""
    shells = []
    lines = [ln.split() for ln in open(path) if ln.strip() and not ln.strip().startswith("*")]
    k = 1  # skip the element line
    while k < len(lines):
        kind, nprim = lines[k][0].lower(), int(lines[k][1])
        if kind not in ("s", "p"):
            raise ValueError(f"{path}: only s and p shells are read, found {kind}")
        prims = [(float(a), float(c)) for a, c in (lines[k + 1 + i][:2] for i in range(nprim))]
        shells.append((kind, prims))
        k += 1 + nprim
    return shells


def pack_shells(shells, prefix):
    """Shells as padded arrays: <prefix>_kind (0 = s, 1 = p), _nprim, _exp, _coef."""
    mp = max(len(p) for _, p in shells)
    exps = np.zeros((len(shells), mp))
    coefs = np.zeros((len(shells), mp))
    for i, (_, prims) in enumerate(shells):
        for j, (a, c) in enumerate(prims):
            exps[i, j], coefs[i, j] = a, c
    return {prefix + "_kind": np.array([0 if k == "s" else 1 for k, _ in shells], dtype=np.int32),
            prefix + "_nprim": np.array([len(p) for _, p in shells], dtype=np.int32),
            prefix + "_exp": exps, prefix + "_coef": coefs}


def h2o():
    d = os.path.join(REF, "tests", "data", "h2o_sto3glibrary_cisd")
    ham = np.loadtxt(os.path.join(d, "cisd_ham_elements.txt"))[:, 0].reshape(141, 141)
    h1 = np.loadtxt(os.path.join(d, "ref_mo_onebody.txt"))
    eri = np.loadtxt(os.path.join(d, "ref_eri.txt"))
    out = os.path.join(HERE, "h2o_sto3g_golden.npz")
    np.savez_compressed(out, cisd_ham=ham, alls_h1=h1, alls_eri=eri)
    print("wrote", out)


def h_minus():
    d = os.path.join(REF, "tests", "data", "PsH_wpos")
    shells = pack_shells(read_g94(os.path.join(d, "electron_basis.g94")), "shell")
    occ = np.loadtxt(os.path.join(d, "h_minus_NO_occ.txt"))
    no = np.loadtxt(os.path.join(d, "h_minus_NO.txt"))
    out = os.path.join(HERE, "h_minus_no_golden.npz")
    np.savez_compressed(out, shell_exp=shells["shell_exp"], shell_coef=shells["shell_coef"],
                        shell_nprim=shells["shell_nprim"], no_occ=occ, no_ao=no)
    print("wrote", out)


def positron_bases():
    """Basis sets of the reference's electron-positron inputs:
    tests/data/li-_custombasis_wpos/Li_basis.g94 (electron and positron basis of Li_wpos.json) and
    tests/data/PsH_wpos/{electron,positron}_basis.g94 (PsH_wpos_CI.json)."""
    li = pack_shells(read_g94(os.path.join(REF, "tests", "data", "li-_custombasis_wpos", "Li_basis.g94")), "li")
    d = os.path.join(REF, "tests", "data", "PsH_wpos")
    pe = pack_shells(read_g94(os.path.join(d, "electron_basis.g94")), "psh_e")
    pp = pack_shells(read_g94(os.path.join(d, "positron_basis.g94")), "psh_p")
    out = os.path.join(HERE, "positron_bases.npz")
    np.savez_compressed(out, **li, **pe, **pp)
    print("wrote", out)


if __name__ == "__main__":
    if not REF or not os.path.isdir(os.path.join(REF, "tests", "data")):
        raise SystemExit("set POLYQUANT_REF to the root of a polyquant source checkout (with tests/data/)")
    h2o()
    h_minus()
    positron_bases()
