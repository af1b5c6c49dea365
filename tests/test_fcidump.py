"""FCIDUMP writer/reader (POLYQUANT_FCIDUMP, src/io/fcidump_utilities.cpp) on CPU."""
import numpy as np

import oracle as O
from cases import batch_dict, h2o_problem, synthetic_ep, synthetic_unrestricted
from polyquant_gb300 import fcidump


def test_header_format():
    h = fcidump.header(7, 10, 0, True, [1] * 14)
    expect = (" &FCI  NORB=     7, NELEC=   10, M2S=    0, \n"
              "  ORBSYM= " + "  1, " * 14 + "\n"
              "    ISYM= 1,\n"
              "    IUHF= 0,\n"
              " PNT_GRP=   C1,\n"
              " &END\n")
    assert h == expect


def test_line_format():
    assert fcidump._line(-74.962926342808259, 0, 0, 0, 0) == (
        "      -74.962926342808260" + "         0" * 4 + "\n")
    assert fcidump._line(0.5, 3, 1, 2, 2) == "        0.500000000000000         3         1         2         2\n"


def test_restricted_round_trip_and_energy(tmp_path, h2o):
    p = h2o_problem(h2o("library"), [2, 2, 4])
    d = batch_dict(p)
    names = fcidump.dump_problem(str(tmp_path / "INTEGRALS"), ["e"], h1=d["h1"], eri=d["eri"], n_part=[10],
                                 ms2=[0], restricted=[1], e_const=p.e_const)
    assert len(names) == 1
    lines = open(names[0]).read().splitlines()
    n = 7
    npair = n * (n + 1) // 2
    # header (6 lines), constant, n orbital energies, lower triangle of h, 4-fold ERI listing
    assert len(lines) == 6 + 1 + n + npair + npair * npair
    r = fcidump.read(names[0])
    assert r["norb"] == 7 and r["nelec"] == 10 and r["ms2"] == 0 and r["restricted"]
    assert abs(r["e_const"] - p.e_const) < 1e-13
    assert np.abs(r["h1"][0] - p.h1[0][0]).max() < 1e-14
    assert np.abs(r["eri"][(0, 0)] - p.eri[(0, 0, 0, 0)]).max() < 1e-14
    kw, ec = fcidump.problem_from_fcidump(names[0], excitation_level=[2, 2, 4])
    q = O.CIProblem(kw["n_orb"], kw["n_alpha"], kw["n_beta"], kw["h1"], kw["eri"], kw["excitation_level"],
                    restricted=kw["restricted"], charge=kw["charge"], e_const=ec)
    a, b = O.Detset(p), O.Detset(q)
    C = np.random.default_rng(0).standard_normal((a.n_dets, 2))
    assert a.n_dets == b.n_dets == 441
    assert np.abs(a.sigma(C) - b.sigma(C)).max() < 1e-11
    w0, w1 = np.linalg.eigvalsh(a.dense_ham())[0], np.linalg.eigvalsh(b.dense_ham())[0]
    assert abs(w0 - w1) < 1e-11


def test_unrestricted_blocks(tmp_path):
    p = synthetic_unrestricted(5, 2, 2, seed=3)
    d = batch_dict(p)
    name = str(tmp_path / "U")
    fcidump.write(name, h1=[p.h1[0][0], p.h1[0][1]],
                  eri={(0, 0): p.eri[(0, 0, 0, 0)], (0, 1): p.eri[(0, 0, 0, 1)], (1, 0): p.eri[(0, 1, 0, 0)],
                       (1, 1): p.eri[(0, 1, 0, 1)]}, restricted=False, n_part=4, ms2=0)
    r = fcidump.read(name)
    assert not r["restricted"]
    for s in range(2):
        assert np.abs(r["h1"][s] - p.h1[0][s]).max() < 1e-14
    assert np.abs(r["eri"][(0, 1)] - p.eri[(0, 0, 0, 1)]).max() < 1e-14
    assert np.abs(r["eri"][(1, 1)] - p.eri[(0, 1, 0, 1)]).max() < 1e-14
    npair = 15
    n_one = sum(1 for ln in open(name).read().splitlines()[6:] if ln.split()[3] == "0" and ln.split()[2] != "0")
    assert n_one == 4 * npair  # spin a's lower triangle once per spin b (as the reference writes it)
    assert d["restricted"] == [0]


def test_cross_species_block(tmp_path):
    p = synthetic_ep(5, 2, 2, 4, 1, 0, seed=3)
    d = batch_dict(p)
    names = fcidump.dump_problem(str(tmp_path / "INTS"), ["electron", "positron"], h1=d["h1"], eri=d["eri"],
                                 n_part=[4, 1], ms2=[0, 1], restricted=[1, 1])
    assert [n.rsplit("/", 1)[-1] for n in names] == ["electron_INTS", "electron_positron_INTS", "positron_INTS"]
    lines = open(names[1]).read().splitlines()
    assert len(lines) == 15 * 10 and not lines[0].lstrip().startswith("&")
    r = fcidump.read(names[1], n_mo_b=4)
    assert np.abs(r["eri"][(0, 0)] - p.eri[(0, 0, 1, 0)]).max() < 1e-14


def test_reads_eightfold_layout(tmp_path):
    """Molpro/pyscf layout: integrals first (unique ij >= kl), constant last."""
    rng = np.random.default_rng(4)
    n = 3
    npair = 6
    M = rng.standard_normal((npair, npair))
    M = M + M.T
    h = rng.standard_normal((n, n))
    h = h + h.T
    txt = " &FCI NORB=3,NELEC=2,MS2=0,\n  ORBSYM=1,1,1,\n  ISYM=1,\n /\n"
    for i in range(n):
        for j in range(i + 1):
            for k in range(n):
                for l in range(k + 1):
                    if fcidump.idx2(i, j) >= fcidump.idx2(k, l):
                        txt += f"{M[fcidump.idx2(i, j), fcidump.idx2(k, l)]:.16e} {i+1} {j+1} {k+1} {l+1}\n"
    for i in range(n):
        for j in range(i + 1):
            txt += f"{h[i, j]:.16e} {i+1} {j+1} 0 0\n"
    txt += "1.25 0 0 0 0\n"
    f = tmp_path / "FCIDUMP"
    f.write_text(txt)
    r = fcidump.read(str(f))
    assert r["norb"] == 3 and r["nelec"] == 2 and r["restricted"]
    assert np.abs(r["eri"][(0, 0)] - M).max() < 1e-15
    assert np.abs(r["h1"][0] - h).max() < 1e-15
    assert r["e_const"] == 1.25
