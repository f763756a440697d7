"""Launch-shape autotuner for batches of small cases.

A batch (hydro_gpu_batch_*) runs each case's step as one branch of a CUDA
graph.  How a case's linear solves are launched decides how well hundreds of
branches share the GPU: grid-wide launches (``cta_threads = 0``: every
sweep and every Krylov iteration is a kernel spread over the SMs) or one CTA
per solve (``cta_threads`` = 256 / 512 / 1024: the whole velocity loop and
the whole pressure solve as one launch that holds one SM).  Small cases
favour the second, large ones the first, and where the crossing lies
depends on the grid size, the thread count and how many cases share the
GPU.  ``tune`` measures it: for every distinct grid size among the cases it
steps a batch of up to ``per_size`` cases of that size under each candidate
shape and keeps the fastest; ``apply`` writes the choices into the
descriptions.  The table (grid size -> choice and the measured times) is
returned so that a run can record what was chosen.

The reference has no counterpart: it runs independent experiments as one
host thread each (source/control/console.cpp:162-178).
"""
import time

from . import capi

CANDIDATES = (0, 256, 512, 1024)


def size_key(desc):
    """Grid size of a case as 'nx x ny[ x nz]'."""
    return "x".join(str(desc.n[k]) for k in range(desc.dim))


def _time_batch(specs, threads, steps, warmup):
    """Seconds per batch step of the cases `specs` [(desc, u0, q0), ...]
    with every case at `threads`, from their initial state."""
    from .solver import Batch
    descs = []
    for d, _, _ in specs:
        d = d.copy()
        d.cta_threads = threads
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
    """specs: [(desc, u0, q0), ...] of the batch.  Returns {size: {"cta_threads":
    best, "ms_per_step": {candidate: ms}, "cases": k}}: for each grid size,
    the first `per_size` cases of that size stepped `warmup` + `steps` batch
    steps under each candidate (host wall clock around the synchronous
    batch steps).  A candidate the cases do not allow (HYDRO_ERR_UNSUPPORTED)
    is skipped."""
    groups = {}
    for s in specs:
        groups.setdefault(size_key(s[0]), []).append(s)
    table = {}
    for key, group in groups.items():
        sample = group[:per_size]
        times = {}
        for t in candidates:
            try:
                times[t] = _time_batch(sample, t, steps, warmup)
            except capi.HydroError as e:
                if e.status != capi.ERR_UNSUPPORTED:
                    raise
        best = min(times, key=times.get)
        table[key] = {"cta_threads": best, "cases": len(sample),
                      "ms_per_step": {str(t): round(v * 1e3, 3) for t, v in times.items()}}
    return table


def apply(descs, table):
    """Sets each description's cta_threads from the table (sizes not in the
    table keep theirs)."""
    for d in descs:
        e = table.get(size_key(d))
        if e is not None:
            d.cta_threads = e["cta_threads"]
    return descs
