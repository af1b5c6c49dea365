"""Host-side loop of calculate_mo_2_body_integrals (integral.cpp:479-516), checked without a GPU by standing in
for the device transform: every species pair b >= a and every spin-block combination is transformed once with
that pair's AO integrals and coefficient blocks; pairs with b < a are left empty."""
import pytest

pytest.importorskip("torch")


def test_blocks_and_arguments(monkeypatch):
    from polyquant_gb300 import integral

    seen = []

    def fake(a, b, Ca, Cb, na, nb, fc, dv, eri, layout, mode):
        seen.append((a, b, Ca, Cb, na, nb, eri))
        return ("T", a, b, Ca, Cb)

    monkeypatch.setattr(integral, "transform_mo_2_body_integrals", fake)
    C = [["e_a"], ["p_a", "p_b"]]  # restricted electrons, unrestricted second species
    eri = {(0, 0): "ee", (0, 1): "ep", (1, 1): "pp"}
    out = integral.calculate_mo_2_body_integrals(C, [1, 0], [0, 0], eri, num_parts=[(2, 2), (1, 1)])
    assert out[0][0][0] == [("T", 0, 0, "e_a", "e_a")]
    assert out[0][0][1] == [("T", 0, 1, "e_a", "p_a"), ("T", 0, 1, "e_a", "p_b")]
    assert out[1][0][0] == [None] and out[1][1][0] == [None]
    assert out[1][1][1] == [("T", 1, 1, "p_b", "p_a"), ("T", 1, 1, "p_b", "p_b")]
    assert len(seen) == 1 + 2 + 4
    assert all(e == {(0, 0): "ee", (0, 1): "ep", (1, 1): "pp"}[(a, b)] for a, b, *_, e in seen)
    assert ("p_b", "p_a", 1, 1) in [(ca, cb, na, nb) for a, b, ca, cb, na, nb, _ in seen if (a, b) == (1, 1)]
