"""FCIDUMP files for the CI integrals: the reference's writer format and a reader.

``write`` reproduces ``POLYQUANT_FCIDUMP::dump`` (src/io/fcidump_utilities.cpp:
18-40) line for line: for a species with itself it writes the header
(:43-63), the constant (:125-132), the orbital energies (:133-153), the lower
triangle of every one-body spin block (:65-86) and the two-body block with
4-fold listing (every pair ij >= ... against every pair ab, :88-123); for two
different species (electron-positron) only the cross two-body block.  File
names follow ``POLYQUANT_EPCI::fcidump`` (src/ci/epci.cpp:528-574):
``<species>_<name>`` and ``<species a>_<species b>_<name>``.

``read`` parses that format and the common Molpro/pyscf layout (integrals
first, 8-fold unique list, constant last) into one-body matrices and
(npair x npair) ERI blocks in the reference layout ``[idx2(i,j), idx2(k,l)]``,
ready for ``POLYQUANT_DETSET``.
"""
from __future__ import annotations

import os
import re
from typing import Dict, List, Optional, Sequence

import numpy as np


def idx2(i: int, j: int) -> int:
    """Pair index of integral.hpp:14-20."""
    return i * (i + 1) // 2 + j if i >= j else j * (j + 1) // 2 + i


def _line(v: float, i: int, j: int, k: int, l: int) -> str:
    return f"{v: >25.15f}{i:>10d}{j:>10d}{k:>10d}{l:>10d}\n"


def header(n_mo: int, n_part: int, ms2: int, restricted: bool, orbsym: Sequence[int], isym: int = 1,
           point_group: str = "C1") -> str:
    """The &FCI namelist exactly as the reference prints it (iostream setw widths)."""
    s = " &FCI  NORB= " + str(n_mo).rjust(5) + ", NELEC= " + str(n_part).rjust(4) + ", M2S= " + str(ms2).rjust(4)
    s += ", \n"
    s += "ORBSYM= ".rjust(10) + "".join(str(x).rjust(3) + ", " for x in orbsym) + "\n"
    s += "ISYM= ".rjust(10) + f"{isym},\n"
    s += "IUHF= ".rjust(10) + f"{0 if restricted else 1},\n"
    s += "PNT_GRP= ".rjust(10) + point_group.rjust(4) + ",\n"
    s += " &END\n"
    return s


def write(filename: str, *, h1: Optional[List[np.ndarray]], eri: Dict, restricted: bool = True,
          n_part: int = 0, ms2: int = 0, e_const: float = 0.0, mo_energy_a=None, mo_energy_b=None,
          same_species: bool = True, orbsym: Optional[Sequence[int]] = None, isym: int = 1,
          point_group: str = "C1") -> None:
    """Write one FCIDUMP block file in the reference's format.

    h1[spin]: (n x n) one-body matrices of the species (same_species only).
    eri[(spin_a, spin_b)]: (npair_a x npair_b) ERI blocks at [idx2(i,j), idx2(a,b)].
    For a species with itself, restricted species need spin 0 only.
    """
    spin_types = 1 if restricted else 2
    out = []
    if same_species:
        n_mo = h1[0].shape[0]
        if orbsym is None:
            # the reference labels MO_a and MO_b columns (both halves, all 1 in C1)
            orbsym = [1] * (2 * n_mo)
        out.append(header(n_mo, n_part, ms2, restricted, orbsym, isym, point_group))
        out.append(_line(e_const, 0, 0, 0, 0))
        ea = np.zeros(n_mo) if mo_energy_a is None else np.asarray(mo_energy_a)
        for i, v in enumerate(ea):
            out.append(_line(float(v), i + 1, 0, 0, 0))
        if spin_types == 2:
            eb = np.zeros(n_mo) if mo_energy_b is None else np.asarray(mo_energy_b)
            for i, v in enumerate(eb):
                out.append(_line(float(v), i + 1, 0, 0, 0))
        for sa in range(spin_types):
            for _sb in range(spin_types):  # the reference repeats spin a's block per spin b
                h = h1[sa]
                for i in range(h.shape[1]):
                    for a in range(i + 1):
                        out.append(_line(float(h[i, a]), i + 1, a + 1, 0, 0))
    for sa in range(spin_types):
        for sb in range(spin_types):
            M = np.asarray(eri[(sa, sb)])
            na = int(round((np.sqrt(8 * M.shape[0] + 1) - 1) / 2))
            nb = int(round((np.sqrt(8 * M.shape[1] + 1) - 1) / 2))
            for i in range(na):
                for j in range(i + 1):
                    row = M[idx2(i, j)]
                    for a in range(nb):
                        for b in range(a + 1):
                            out.append(_line(float(row[idx2(a, b)]), i + 1, j + 1, a + 1, b + 1))
    with open(filename, "w") as f:
        f.write("".join(out))


def dump_problem(basename: str, species: Sequence[str], *, h1, eri: Dict, n_part: Sequence[int],
                 ms2: Sequence[int], restricted: Sequence[int], e_const: float = 0.0, mo_energy=None) -> List[str]:
    """All block files of a CI problem as ``POLYQUANT_EPCI::fcidump`` names them.

    h1[s][spin], eri[(a, sa, b, sb)] as for ``POLYQUANT_DETSET``; returns the file names written."""
    names = []
    ns = len(species)
    folder, base = os.path.split(basename)
    for a in range(ns):
        ra = bool(restricted[a])
        st = 1 if ra else 2
        for b in range(a, ns):
            blocks = {}
            for sa in range(st):
                for sb in range(st):
                    key = (a, sa, b, sb if b == a or not restricted[b] else 0)
                    if key not in eri and a == b:
                        key = (a, sb, a, sa)
                        blocks[(sa, sb)] = np.asarray(eri[key]).T
                    else:
                        blocks[(sa, sb)] = np.asarray(eri[key])
            if a == b:
                name = os.path.join(folder, f"{species[a]}_{base}")
                me = None if mo_energy is None else mo_energy[a]
                write(name, h1=[np.asarray(h1[a][s % len(h1[a])]) for s in range(st)], eri=blocks, restricted=ra,
                      n_part=n_part[a], ms2=ms2[a], e_const=e_const,
                      mo_energy_a=None if me is None else me[0],
                      mo_energy_b=None if me is None else me[-1])
            else:
                name = os.path.join(folder, f"{species[a]}_{species[b]}_{base}")
                write(name, h1=None, eri=blocks, restricted=ra, same_species=False)
            names.append(name)
    return names


_KEY = re.compile(r"([A-Za-z_0-9]+)\s*=\s*([^=]*?)(?=,?\s*[A-Za-z_0-9]+\s*=|/|&END|$)", re.S)


def read(filename: str, n_mo_b: Optional[int] = None) -> dict:
    """Parse an FCIDUMP.  Returns {"header": {...}, "norb", "nelec", "ms2", "restricted", "e_const",
    "mo_energy": [per spin], "h1": [per spin], "eri": {(sa, sb): matrix}}.

    Spin blocks are mapped by their order in the file (alpha first), as the reference writes them; a
    cross-species file has no header and needs n_mo_b (the second species' orbital count) only when
    it cannot be inferred from the largest index."""
    with open(filename) as f:
        text = f.read()
    hdr = {}
    body = text
    m = re.search(r"&FCI(.*?)(&END|/)", text, re.S | re.I)
    if m:
        for k, v in _KEY.findall(m.group(1)):
            hdr[k.upper()] = v.strip().rstrip(",").strip()
        body = text[m.end():]
    rows = []
    for ln in body.splitlines():
        p = ln.split()
        if len(p) != 5:
            continue
        rows.append((float(p[0].replace("D", "E").replace("d", "e")), int(p[1]), int(p[2]), int(p[3]), int(p[4])))
    norb = int(hdr["NORB"]) if "NORB" in hdr else max(max(r[1], r[2]) for r in rows)
    nelec = int(hdr.get("NELEC", 0))
    ms2 = int(hdr.get("MS2", hdr.get("M2S", 0)))
    uhf = hdr.get("IUHF", hdr.get("UHF", "0")).upper() in ("1", ".TRUE.", "TRUE", "T")
    st = 2 if uhf else 1
    res = {"header": hdr, "norb": norb, "nelec": nelec, "ms2": ms2, "restricted": not uhf, "e_const": 0.0}
    np_a = norb * (norb + 1) // 2
    if not m:
        # cross-species block: 4-fold listing, no one-body part
        nb = n_mo_b or max(r[3] for r in rows)
        npb = nb * (nb + 1) // 2
        M = np.zeros((np_a, npb))
        for v, i, j, k, l in rows:
            M[idx2(i - 1, j - 1), idx2(k - 1, l - 1)] = v
        res["eri"] = {(0, 0): M}
        res["h1"] = None
        return res
    mo = [[] for _ in range(st)]
    h1 = [np.zeros((norb, norb)) for _ in range(st)]
    eri = {}
    one = [r for r in rows if r[3] == 0 and r[1] > 0 and r[2] > 0]
    two = [r for r in rows if r[3] > 0]
    for v, i, j, k, l in rows:
        if i == 0 and j == 0 and k == 0 and l == 0:
            res["e_const"] = v
    energies = [r for r in rows if r[1] > 0 and r[2] == 0 and r[3] == 0]
    for n, r in enumerate(energies):
        mo[min(n // norb, st - 1)].append(r[0])
    # one-body: tri = norb(norb+1)/2 lines per listed block; the reference lists spin a's block st times
    tri = np_a
    nblk = max(1, len(one) // tri)
    for bi in range(nblk):
        s = min(bi * st // nblk, st - 1)
        for v, i, j, _, _ in one[bi * tri:(bi + 1) * tri]:
            h1[s][i - 1, j - 1] = h1[s][j - 1, i - 1] = v
    # two-body: 4-fold (np_a^2 lines per block, reference) or 8-fold (unique pairs, Molpro/pyscf)
    full4 = np_a * np_a
    if len(two) >= full4 and len(two) % full4 == 0:
        nblk = len(two) // full4
        for bi in range(nblk):
            sa, sb = (bi // st, bi % st) if nblk == st * st else (0, 0)
            M = np.zeros((np_a, np_a))
            for v, i, j, k, l in two[bi * full4:(bi + 1) * full4]:
                M[idx2(i - 1, j - 1), idx2(k - 1, l - 1)] = v
            eri[(sa, sb)] = M
    else:
        M = np.zeros((np_a, np_a))
        for v, i, j, k, l in two:
            p, q = idx2(i - 1, j - 1), idx2(k - 1, l - 1)
            M[p, q] = M[q, p] = v
        eri[(0, 0)] = M
    res["h1"] = h1
    res["mo_energy"] = [np.array(x) for x in mo]
    res["eri"] = eri
    return res


def problem_from_fcidump(filename: str, excitation_level=None) -> dict:
    """Keyword arguments of ``POLYQUANT_DETSET`` for a single-species FCIDUMP (full CI by default)."""
    d = read(filename)
    n, ne, ms2 = d["norb"], d["nelec"], d["ms2"]
    na, nb = (ne + ms2) // 2, (ne - ms2) // 2
    if excitation_level is None:
        excitation_level = [min(na, n - na), min(nb, n - nb), min(na, n - na) + min(nb, n - nb)]
    eri = {(0, 0, 0, 0): d["eri"][(0, 0)]}
    h1 = [d["h1"][0]] if d["restricted"] else d["h1"]
    if not d["restricted"]:
        eri[(0, 0, 0, 1)] = d["eri"][(0, 1)]
        eri[(0, 1, 0, 1)] = d["eri"][(1, 1)]
    return dict(n_orb=[n], n_alpha=[na], n_beta=[nb], h1=[h1], eri=eri, excitation_level=[excitation_level],
                restricted=[1 if d["restricted"] else 0], charge=[-1.0]), d["e_const"]
