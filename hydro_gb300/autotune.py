"""Launch-shape autotuner for batches of small cases.

A batch (hydro_gpu_batch_*) runs each case's step as one branch of a CUDA
graph.  How a case's linear solves are launched decides how well hundreds of
branches share the GPU: grid-wide launches (``cta_threads = 0``: every
sweep and every Krylov iteration is a kernel spread over the SMs), one CTA
per solve (``cta_threads`` = 512 / 1024: the whole velocity loop and the
whole pressure solve as one launch that holds one SM) or one thread-block
cluster per solve (``cta_cluster`` = 2 / 4 / 8 such CTAs on as many SMs).
Small cases favour the one-CTA form, larger ones a cluster or the grid,
and where the crossings lie depends on the grid size, the shape and how
many cases share the GPU.  ``tune`` measures it: for every distinct grid
size among the cases it steps a batch of up to ``per_size`` cases of that
size under each candidate shape and keeps the fastest; ``apply`` writes the
choices into the descriptions.  The table (grid size -> choice and the
measured times) is returned so that a run can record what was chosen.

The reference has no counterpart: it runs independent experiments as one
host thread each (source/control/console.cpp:162-178).
"""
import time

from . import capi

# (cta_threads, cta_cluster): grid launches, one CTA, clusters of 2/4/8 CTAs
CANDIDATES = ((0, 0), (512, 1), (1024, 1), (1024, 2), (1024, 4), (1024, 8))


def _name(shape):
    t, c = shape
    return "grid" if t == 0 else ("cta%d" % t if c <= 1 else "cta%dx%d" % (t, c))


def size_key(desc):
    """Grid size of a case as 'nx x ny[ x nz]'."""
    return "x".join(str(desc.n[k]) for k in range(desc.dim))


def _time_batch(specs, shape, steps, warmup):
    """Seconds per batch step of the cases `specs` [(desc, u0, q0), ...]
    with every case in the launch shape (cta_threads, cta_cluster), from
    their initial state."""
    from .solver import Batch
    descs = []
    for d, _, _ in specs:
        d = d.copy()
        d.cta_threads, d.cta_cluster = shape
        descs.append(d)
    b = Batch(descs)
    try:
        for c, (_, u0, q0) in zip(b.cases, specs):
            c.set_field(capi.F_VELOCITY, u0)
            c.set_field(capi.F_PARTIAL_DENSITY, q0)
        b.init_state()
        for _ in range(warmup):
            b.step()
        t0 = time.perf_counter()
        for _ in range(steps):
            b.step()  # waits for the batch's graph launch
        return (time.perf_counter() - t0) / steps
    finally:
        b.close()


def tune(specs, per_size=24, steps=2, warmup=1, candidates=CANDIDATES):
    """specs: [(desc, u0, q0), ...] of the batch.  Returns {size:
    {"cta_threads": t, "cta_cluster": c, "shape": name, "ms_per_step":
    {name: ms}, "cases": k}}: for each grid size, the first `per_size` cases
    of that size stepped `warmup` + `steps` batch steps under each candidate
    shape (host wall clock around the synchronous batch steps).  A shape
    the cases do not allow (HYDRO_ERR_UNSUPPORTED) is skipped."""
    groups = {}
    for s in specs:
        groups.setdefault(size_key(s[0]), []).append(s)
    table = {}
    for key, group in groups.items():
        sample = group[:per_size]
        times = {}
        for shape in candidates:
            try:
                times[shape] = _time_batch(sample, shape, steps, warmup)
            except capi.HydroError as e:
                if e.status != capi.ERR_UNSUPPORTED:
                    raise
        best = min(times, key=times.get)
        table[key] = {"cta_threads": best[0], "cta_cluster": best[1], "shape": _name(best),
                      "cases": len(sample),
                      "ms_per_step": {_name(t): round(v * 1e3, 3) for t, v in times.items()}}
    return table


def apply(descs, table):
    """Sets each description's cta_threads from the table (sizes not in the
    table keep theirs)."""
    for d in descs:
        e = table.get(size_key(d))
        if e is not None:
            d.cta_threads = e["cta_threads"]
            d.cta_cluster = e["cta_cluster"]
    return descs
