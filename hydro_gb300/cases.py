"""Case builders: the .hydroconf keys and initial fields of the workloads.

Each builder returns ``(desc, u0, q0)``: a ``capi.HydroDesc``, the initial
velocity (component-major, cells in the reference raw order) and the initial
partial densities (phase-major).  Initial fields follow hydro<Mesh>'s
initialisation (hydro2d.hpp:476-566): phase 1 occupies a region, its partial
density is smoothed ``initial_volume_fraction_smooth_times`` times with
GetSmoothField, and phase 0 compensates, q0 = (1 - q1/rho1) * rho0.

Workloads stand in for the reference's example cases with seeded synthetic
inputs of the stated shapes (no external data):
  cavity         lid-driven cavity (examples/cavity)
  broken_dam     two-phase dam break (examples/broken_dam_2d)
  rayleigh_taylor 3D RT with a seeded 16-mode Fourier interface
  rising_drops   3D drops, 1-8 seeded spheres
"""
import numpy as np

from . import capi


def cell_centers(desc):
    """Cell centres, arrays of shape (ncells,) per dimension, raw order."""
    dim = desc.dim
    n = [desc.n[k] if k < dim else 1 for k in range(3)]
    h = [(desc.hi[k] - desc.lo[k]) / n[k] if k < dim else 1.0 for k in range(3)]
    k, j, i = np.meshgrid(np.arange(n[2]), np.arange(n[1]), np.arange(n[0]), indexing="ij")
    xs = [desc.lo[0] + (i.ravel() + 0.5) * h[0], desc.lo[1] + (j.ravel() + 0.5) * h[1]]
    if dim == 3:
        xs.append(desc.lo[2] + (k.ravel() + 0.5) * h[2])
    return xs


def smooth(desc, field, repeat):
    """GetSmoothField (solver.hpp:636-656): face averages with
    zero-derivative boundaries, then the average of the 2*dim faces."""
    dim = desc.dim
    shape = tuple(desc.n[k] for k in reversed(range(dim)))  # (z,) y, x
    a = np.asarray(field, dtype=np.float64).reshape(shape).copy()
    for _ in range(repeat):
        acc = np.zeros_like(a)
        for ax in range(dim):
            # faces along axis ax: boundary faces carry the cell value
            lo = np.concatenate([a.take([0], axis=ax), (a.take(range(0, a.shape[ax] - 1), axis=ax) * 0.5 +
                                                        a.take(range(1, a.shape[ax]), axis=ax) * 0.5)], axis=ax)
            hi = np.concatenate([(a.take(range(0, a.shape[ax] - 1), axis=ax) * 0.5 +
                                  a.take(range(1, a.shape[ax]), axis=ax) * 0.5), a.take([a.shape[ax] - 1], axis=ax)], axis=ax)
            acc_ax = lo + hi
            acc = acc + acc_ax if ax else acc_ax
        a = acc / (2 * dim)
    return a.ravel()


def two_phase_q(desc, alpha1, smooth_times):
    rho0, rho1 = desc.density[0], desc.density[1]
    q1 = smooth(desc, alpha1 * rho1, smooth_times)
    q0 = (1.0 - q1 / rho1) * rho0
    return np.concatenate([q0, q1])


def _common(desc):
    desc.velocity_solver = capi.LINEAR_JACOBI
    desc.pressure_solver = capi.LINEAR_CG
    return desc


def cavity(n=64, mu=0.01, dt=1e-3, lid=1.0, dim=2, steps_hint=200):
    """Lid-driven cavity: unit square (cube), walls, lid velocity (lid, 0)."""
    d = capi.default_desc()
    d.dim = dim
    for k in range(3):
        d.n[k] = n
        d.lo[k], d.hi[k] = 0.0, 1.0
    top = capi.YP if dim == 2 else capi.ZP
    if dim == 2:
        d.bc_velocity[capi.YP][0] = lid
    else:
        # lid on the top (y-high) wall, moving along x
        d.bc_velocity[capi.YP][0] = lid
    del top
    d.dt = dt
    d.num_phases = 1
    d.density[0] = 1.0
    d.viscosity[0] = mu
    d.advection_enable = 0
    d.convergence_tolerance = 1e-8
    d.num_iterations_limit = 20
    _common(d)
    nc = d.ncells
    u0 = np.zeros(nc * dim)
    q0 = np.ones(nc) * d.density[0]
    return d, u0, q0


def broken_dam(nx=512, ny=256, dt_auto=True, dt=1e-3, cfl=0.25, dt_max=1e-3,
               smooth_times=0):
    """Two-phase broken dam: domain 4x2, heavy phase in [0,1]x[0,1.5]."""
    d = capi.default_desc()
    d.dim = 2
    d.n[0], d.n[1] = nx, ny
    d.lo[0], d.lo[1] = 0.0, 0.0
    d.hi[0], d.hi[1] = 4.0, 2.0
    d.num_phases = 2
    d.density[0], d.viscosity[0] = 1.0, 1e-5
    d.density[1], d.viscosity[1] = 1000.0, 1e-3
    d.gravity[1] = -9.81
    d.dt = dt
    d.dt_auto = 1 if dt_auto else 0
    d.cfl = cfl
    d.cfl_advection = cfl
    d.dt_max = dt_max
    d.convergence_tolerance = 1e-8
    d.num_iterations_limit = 20
    _common(d)
    x, y = cell_centers(d)
    alpha1 = ((x > 0.0) & (x < 1.0) & (y > 0.0) & (y < 1.5)).astype(np.float64)
    q0 = two_phase_q(d, alpha1, smooth_times)
    u0 = np.zeros(d.ncells * 2)
    return d, u0, q0


def rayleigh_taylor(nx=128, ny=128, nz=512, seed=0, dt_auto=True, cfl=0.25,
                    dt_max=1e-2, sub=8):
    """3D Rayleigh-Taylor in 1x1x4: heavy (3) over light (1), mu 1e-3,
    g = -1 along z; interface z = 2 + eta(x, y), eta a sum of 16 seeded
    Fourier modes with integer wavevectors 1 <= |k| <= 8, amplitudes
    U[0, 1e-2], phases U[0, 2pi).  Volume fraction is the cell average of
    the Heaviside function over sub^3 samples."""
    d = capi.default_desc()
    d.dim = 3
    d.n[0], d.n[1], d.n[2] = nx, ny, nz
    for k in range(3):
        d.lo[k] = 0.0
    d.hi[0], d.hi[1], d.hi[2] = 1.0, 1.0, 4.0
    d.num_phases = 2
    d.density[0], d.viscosity[0] = 1.0, 1e-3
    d.density[1], d.viscosity[1] = 3.0, 1e-3
    d.gravity[2] = -1.0
    d.dt_auto = 1 if dt_auto else 0
    d.cfl = cfl
    d.cfl_advection = cfl
    d.dt_max = dt_max
    d.dt = dt_max
    d.convergence_tolerance = 1e-8
    d.num_iterations_limit = 20
    _common(d)
    rng = np.random.Generator(np.random.Philox(seed))
    modes = []
    while len(modes) < 16:
        kx, ky = rng.integers(-8, 9, size=2)
        kk = np.hypot(kx, ky)
        if 1 <= kk <= 8:
            modes.append((kx, ky, rng.uniform(0, 1e-2), rng.uniform(0, 2 * np.pi)))
    hx, hy, hz = 1.0 / nx, 1.0 / ny, 4.0 / nz
    # subsample the Heaviside per column; eta depends on (x, y) only
    alpha = np.zeros((nz, ny, nx))
    offs = (np.arange(sub) + 0.5) / sub
    zc = (np.arange(nz) + 0.5) * hz
    for sx in offs:
        for sy in offs:
            X, Y = np.meshgrid((np.arange(nx) + sx) * hx, (np.arange(ny) + sy) * hy)
            eta = np.zeros_like(X)
            for kx, ky, a, ph in modes:
                eta += a * np.cos(2 * np.pi * (kx * X + ky * Y) + ph)
            zi = 2.0 + eta  # (ny, nx)
            for sz in offs:
                zs = (np.arange(nz) + sz) * hz
                alpha += (zs[:, None, None] > zi[None, :, :])
    del zc
    alpha /= sub ** 3
    q0 = two_phase_q(d, alpha.ravel(), 0)
    u0 = np.zeros(d.ncells * 3)
    return d, u0, q0


def rising_drops(n=192, seed=0, dt_auto=True, cfl=0.25, dt_max=2e-3,
                 smooth_times=2):
    """3D rising drops in the unit cube: ambient rho 10 / mu 1e-2 (phase 0),
    drops rho 1 / mu 1e-2 (phase 1), g = -1 along z.  Per seed: 1-8 spheres,
    radius U[0.04, 0.12], centres rejection-sampled in [r, 1-r]^3 without
    overlap.  A cell is inside when its centre is (hydro2d.hpp:545-556)."""
    d = capi.default_desc()
    d.dim = 3
    for k in range(3):
        d.n[k] = n
        d.lo[k], d.hi[k] = 0.0, 1.0
    d.num_phases = 2
    d.density[0], d.viscosity[0] = 10.0, 1e-2
    d.density[1], d.viscosity[1] = 1.0, 1e-2
    d.gravity[2] = -1.0
    d.dt_auto = 1 if dt_auto else 0
    d.cfl = cfl
    d.cfl_advection = cfl
    d.dt_max = dt_max
    d.dt = dt_max
    d.convergence_tolerance = 1e-8
    d.num_iterations_limit = 20
    _common(d)
    rng = np.random.Generator(np.random.Philox(seed))
    count = int(rng.integers(1, 9))
    drops = []
    tries = 0
    while len(drops) < count and tries < 10000:
        tries += 1
        r = rng.uniform(0.04, 0.12)
        c = rng.uniform(r, 1 - r, size=3)
        if all(np.linalg.norm(c - c2) > r + r2 for c2, r2 in drops):
            drops.append((c, r))
    x, y, z = cell_centers(d)
    alpha1 = np.zeros(d.ncells)
    for c, r in drops:
        inside = (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2 < r * r
        alpha1[inside] = 1.0
    q0 = two_phase_q(d, alpha1, smooth_times)
    u0 = np.zeros(d.ncells * 3)
    return d, u0, q0, drops


def cavity_batch(ncases=512, seed=0, sizes=(64, 96, 128, 192, 256), dt=1e-3):
    """Independent 2D lid-driven cavities of uneven size: per case the grid
    size is drawn uniformly from `sizes`, Re = exp(U[ln 100, ln 5000]) and
    mu = 1/Re (rho = 1, unit square, lid velocity 1), dt pinned.  Seeded
    (Philox).  Returns a list of (desc, u0, q0, Re)."""
    rng = np.random.Generator(np.random.Philox(seed))
    out = []
    for _ in range(ncases):
        n = int(sizes[rng.integers(len(sizes))])
        re = float(np.exp(rng.uniform(np.log(100.0), np.log(5000.0))))
        d, u0, q0 = cavity(n=n, mu=1.0 / re, dt=dt, lid=1.0)
        out.append((d, u0, q0, re))
    return out


def channel(nx=40, ny=20, nz=1, dim=2, length=2.0, u_in=1.0, mu=0.01, dt=1e-2, reverse=False,
            two_phase=False):
    """Channel flow: inlet on one x side with velocity (u_in, 0[, 0]) into
    the domain, outlet on the other (rebalanced to the inflow), walls
    elsewhere; starts at rest.  With two_phase, phase 1 (rho 2, mu 2 mu)
    fills the inlet half of the channel below y = 0.5 and the inlet faces
    inject it; phase 0 has rho 1."""
    d = capi.default_desc()
    d.dim = dim
    n = (nx, ny, nz if dim == 3 else 1)
    hi = (length, 1.0, 1.0)
    for k in range(3):
        d.n[k] = n[k]
        d.lo[k], d.hi[k] = 0.0, hi[k]
    inlet, outlet = (capi.XP, capi.XM) if reverse else (capi.XM, capi.XP)
    d.bc_kind[inlet] = capi.BC_INLET
    d.bc_kind[outlet] = capi.BC_OUTLET
    d.bc_velocity[inlet][0] = -u_in if reverse else u_in
    d.dt = dt
    d.num_phases = 2 if two_phase else 1
    d.density[0], d.viscosity[0] = 1.0, mu
    d.density[1], d.viscosity[1] = 2.0, 2 * mu
    d.advection_enable = 1 if two_phase else 0
    d.gravity[0] = d.gravity[1] = d.gravity[2] = 0.0
    _common(d)
    nc = d.ncells
    u0 = np.zeros(nc * dim)
    if two_phase:
        x, y = cell_centers(d)[:2]
        near = (x > length / 2) if reverse else (x < length / 2)
        alpha1 = (near & (y < 0.5)).astype(float)
        q0 = two_phase_q(d, alpha1, 0)
    else:
        q0 = np.ones(nc) * d.density[0]
    return d, u0, q0


def hydrostatic_pressure(desc, rho):
    """Pressure in hydrostatic balance with the cell density rho (raw order)
    for gravity along one axis: dp/dx_a = rho g_a integrated cell to cell
    with the face density (the mean of the two cells), zero mean.  The
    fluid at rest then starts without the one-off pressure build-up of its
    first step.  Zeros when gravity is zero or not along one axis."""
    dim = desc.dim
    g = [desc.gravity[k] for k in range(dim)]
    axes = [k for k in range(dim) if g[k] != 0.0]
    shape = tuple(desc.n[k] for k in reversed(range(dim)))
    if len(axes) != 1:
        return np.zeros(int(np.prod(shape)))
    a = axes[0]
    ax = dim - 1 - a  # numpy axis of direction a (arrays are (z,) y, x)
    r = np.asarray(rho, dtype=np.float64).reshape(shape)
    h = (desc.hi[a] - desc.lo[a]) / desc.n[a]
    face = 0.5 * (r.take(range(1, shape[ax]), axis=ax) + r.take(range(0, shape[ax] - 1), axis=ax))
    inc = np.cumsum(face * (g[a] * h), axis=ax)
    p = np.concatenate([np.zeros_like(r.take([0], axis=ax)), inc], axis=ax)
    return (p - p.mean()).ravel()
