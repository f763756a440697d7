"""Host logic of the launch-shape autotuner without a GPU: cases grouped by
grid size, the fastest candidate kept per size, shapes a case refuses
(HYDRO_ERR_UNSUPPORTED) skipped, other errors raised, and the choices
written back into the descriptions."""
import pytest

from hydro_gb300 import autotune, capi, cases


def _specs(sizes):
    out = []
    for n in sizes:
        d, u0, q0 = cases.cavity(n=n, mu=1e-2, dt=1e-3)
        out.append((d, u0, q0))
    return out


def test_size_key():
    d, _, _ = cases.cavity(n=96, mu=1e-2, dt=1e-3)
    assert autotune.size_key(d) == "96x96"


def test_tune_keeps_the_fastest_shape_per_size(monkeypatch):
    calls = []
    # a made-up cost model: one CTA is best at 64^2, a 4-CTA cluster at
    # 128^2; 8-CTA clusters are refused at 64^2
    cost = {("64x64", (0, 0)): 9.0, ("64x64", (512, 1)): 5.0, ("64x64", (1024, 1)): 6.0,
            ("64x64", (1024, 2)): 6.5, ("64x64", (1024, 4)): 7.0,
            ("128x128", (0, 0)): 20.0, ("128x128", (512, 1)): 30.0,
            ("128x128", (1024, 1)): 25.0, ("128x128", (1024, 2)): 18.0,
            ("128x128", (1024, 4)): 15.0, ("128x128", (1024, 8)): 17.0}

    def fake_time(specs, shape, steps, warmup):
        key = autotune.size_key(specs[0][0])
        assert all(autotune.size_key(s[0]) == key for s in specs)
        calls.append((key, shape, len(specs)))
        if (key, shape) not in cost:
            raise capi.HydroError(capi.ERR_UNSUPPORTED, "test")
        return cost[(key, shape)] / 1e3

    monkeypatch.setattr(autotune, "_time_batch", fake_time)
    specs = _specs([64, 128, 64, 128, 64])
    table = autotune.tune(specs, per_size=2)
    assert set(table) == {"64x64", "128x128"}
    assert (table["64x64"]["cta_threads"], table["64x64"]["cta_cluster"]) == (512, 1)
    assert table["64x64"]["shape"] == "cta512"
    assert "cta1024x8" not in table["64x64"]["ms_per_step"]  # refused, skipped
    assert (table["128x128"]["cta_threads"], table["128x128"]["cta_cluster"]) == (1024, 4)
    assert table["128x128"]["ms_per_step"]["cta1024x4"] == 15.0
    # at most per_size cases of each size are stepped, every candidate once
    assert all(k <= 2 for _, _, k in calls)
    assert len(calls) == 2 * len(autotune.CANDIDATES)

    descs = [s[0].copy() for s in specs]
    autotune.apply(descs, table)
    assert [(d.cta_threads, d.cta_cluster) for d in descs] == [
        (512, 1), (1024, 4), (512, 1), (1024, 4), (512, 1)]


def test_tune_raises_other_errors(monkeypatch):
    def fake_time(specs, shape, steps, warmup):
        raise capi.HydroError(capi.ERR_CUDA, "test")

    monkeypatch.setattr(autotune, "_time_batch", fake_time)
    with pytest.raises(capi.HydroError):
        autotune.tune(_specs([64]))


def test_apply_keeps_sizes_not_in_the_table():
    specs = _specs([64, 96])
    descs = [s[0].copy() for s in specs]
    descs[1].cta_threads, descs[1].cta_cluster = 256, 1
    autotune.apply(descs, {"64x64": {"cta_threads": 1024, "cta_cluster": 8}})
    assert (descs[0].cta_threads, descs[0].cta_cluster) == (1024, 8)
    assert (descs[1].cta_threads, descs[1].cta_cluster) == (256, 1)
