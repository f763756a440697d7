"""Seeded synthetic case generators (CPU): shapes, ranges and determinism."""
import numpy as np
import pytest

from hydro_gb300 import cases


def test_batch_cavity_sizes_and_reynolds():
    """The many-cavity generator draws sizes from the given set and Re in
    [100, 5000] with mu = 1/Re."""
    cs = cases.cavity_batch(ncases=64, seed=0)
    sizes = {d.n[0] for d, _, _, _ in cs}
    assert sizes <= {64, 96, 128, 192, 256} and len(sizes) >= 4
    for d, _, _, re in cs:
        assert 100.0 <= re <= 5000.0
        assert d.viscosity[0] == pytest.approx(1.0 / re)
        assert d.n[0] == d.n[1] and d.dt == 1e-3


def test_cavity_batch_is_seeded():
    a = cases.cavity_batch(ncases=8, seed=3)
    b = cases.cavity_batch(ncases=8, seed=3)
    assert [(d.n[0], re) for d, _, _, re in a] == [(d.n[0], re) for d, _, _, re in b]
    c = cases.cavity_batch(ncases=8, seed=4)
    assert [re for *_, re in a] != [re for *_, re in c]


def test_rising_drops_fraction_bounds():
    d, u0, q0, drops = cases.rising_drops(n=16, seed=5)
    assert 1 <= len(drops) <= 8
    assert np.all(np.isfinite(q0)) and np.all(u0 == 0)
