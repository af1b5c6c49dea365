"""QMCPACK multideterminant payload of a CI solution.

Restates the data of POLYQUANT_CALCULATION::dump_post_mf_for_qmcpack
(src/calculation/calculation.cpp:625-660) and
POLYQUANT_HDF5::dump_post_mf_to_hdf5_for_QMCPACK (src/io/hdf5_utilities.cpp:399-467),
the datasets of the /MultiDet group:

  CI_<2 * species + spin>  N_dets x Nbits uint64: the determinant's string of
                           that species and spin with the frozen-core orbitals
                           put back (get_det_withfcorbs,
                           src/ci/detset/determinant_creation.cpp:391-454:
                           active orbital o becomes o + n_frozen, orbitals
                           0..n_frozen-1 occupied), word j holding orbitals
                           64 j .. 64 j + 63 (the reference's word order
                           reversed, as the writer stores it)
  Coeff, Coeff_1, ...      the CI vector of each state
  NbDet                    N_dets
  Nbits                    words per string: (max over species of active +
                           frozen orbitals >> 6) + 1
  nexcitedstate            number of states
  nstate                   max over species of active + frozen orbitals

``multidet_payload`` returns them as numpy arrays keyed by dataset name;
``write_multidet`` stores them under /MultiDet of an HDF5 file with h5py.  The
HDF5 format itself is not written here: without h5py the call raises, unless
the caller asks for an .npz archive with the same keys (``allow_npz=True``).
"""
from __future__ import annotations

from typing import Dict, Optional, Sequence

import numpy as np


def strings_with_frozen_core(masks: np.ndarray, n_frozen: int, n_words: int) -> np.ndarray:
    """Active-space occupation masks (uint64, bit o = active orbital o, < 64 orbitals) -> (n, n_words) words of
    the full-orbital string with orbitals 0..n_frozen-1 occupied, word j = orbitals 64 j .. 64 j + 63."""
    if n_frozen < 0 or n_frozen >= 64:
        raise ValueError("0 <= n_frozen < 64 frozen orbitals supported")  # the reference aborts at > 64
    m = np.asarray(masks, dtype=np.uint64)
    out = np.zeros((m.shape[0], n_words), dtype=np.uint64)
    if n_frozen == 0:
        out[:, 0] = m
        return out
    sh = np.uint64(n_frozen)
    out[:, 0] = (m << sh) | np.uint64((1 << n_frozen) - 1)
    spill = m >> np.uint64(64 - n_frozen)
    if n_words > 1:
        out[:, 1] = spill
    elif np.any(spill):
        raise ValueError("strings with frozen orbitals need more than one 64-bit word")
    return out


def multidet_payload(strings: Sequence[Sequence[np.ndarray]], unfold: np.ndarray, C: np.ndarray,
                     n_orb: Sequence[int], frozen_core: Optional[Sequence[int]] = None) -> Dict[str, np.ndarray]:
    """/MultiDet datasets from the string lists, the determinant unfold table and the CI vectors.

    strings[s][spin]  uint64 occupation masks of species s (reference string order)
    unfold            (N_dets, 2 * n_species) string indices of every determinant (det_idx_unfold)
    C                 (N_dets, n_states) CI vectors
    n_orb             active orbitals per species
    """
    ns = len(strings)
    fc = list(frozen_core) if frozen_core is not None else [0] * ns
    C = np.asarray(C, dtype=np.float64).reshape(unfold.shape[0], -1)
    n_mo = max(n_orb[s] + fc[s] for s in range(ns))
    n_words = (n_mo >> 6) + 1
    out: Dict[str, np.ndarray] = {}
    for s in range(ns):
        for spin in range(2):
            masks = np.asarray(strings[s][spin], dtype=np.uint64)[unfold[:, 2 * s + spin]]
            out[f"CI_{2 * s + spin}"] = strings_with_frozen_core(masks, fc[s], n_words)
    for i in range(C.shape[1]):
        out["Coeff" if i == 0 else f"Coeff_{i}"] = np.ascontiguousarray(C[:, i])
    out["NbDet"] = np.array(unfold.shape[0], dtype=np.int64)
    out["Nbits"] = np.array(n_words, dtype=np.int64)
    out["nexcitedstate"] = np.array(C.shape[1], dtype=np.int64)
    out["nstate"] = np.array(n_mo, dtype=np.int64)
    return out


def multidet_payload_from_detset(ds, C_ci, frozen_core: Optional[Sequence[int]] = None) -> Dict[str, np.ndarray]:
    """The payload of a POLYQUANT_DETSET and its CI vectors (torch CUDA or numpy, N_dets x n_states)."""
    strings = [[_masks(ds.strings(s, spin)) for spin in range(2)] for s in range(ds.n_species)]
    C = C_ci.detach().cpu().numpy() if hasattr(C_ci, "detach") else np.asarray(C_ci)
    return multidet_payload(strings, ds.det_unfold(), C, ds.n_orb, frozen_core)


def _masks(words: np.ndarray) -> np.ndarray:
    """(n, n_words) strings in the reference word layout (last word = orbitals 0..63) -> uint64 masks."""
    w = np.asarray(words, dtype=np.uint64)
    return w[:, -1] if w.ndim == 2 else w


def write_multidet(path: str, payload: Dict[str, np.ndarray], allow_npz: bool = False) -> str:
    """Store the payload under /MultiDet of the HDF5 file ``path`` (needs h5py).  Without h5py this raises
    RuntimeError, or, with ``allow_npz=True``, writes ``path`` + '.npz' with the same dataset names.
    Returns the file written."""
    try:
        import h5py
    except ImportError:
        if not allow_npz:
            raise RuntimeError("write_multidet: writing the QMCPACK HDF5 file needs h5py, which is not installed; "
                               "pass allow_npz=True to store the /MultiDet datasets as an .npz archive instead")
        out = path + ".npz"
        np.savez(out, **payload)
        return out
    with h5py.File(path, "a") as f:
        g = f.require_group("MultiDet")
        for k, v in payload.items():
            if k in g:
                del g[k]
            g.create_dataset(k, data=v)
    return path
