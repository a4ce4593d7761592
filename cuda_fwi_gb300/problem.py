"""Host-side description of an FWI problem in the reference's conventions.

A ``Problem`` holds everything the reference's ``FDWaveModel`` assembles before
it calls the propagators (Mohammad-debug/CUDA_FWI, CUDA_week2/fd_wave_model.cu:33-75):
the padded grid (fd_grid.cu:52-71), Holberg coefficients (holbergcoeff.cu),
CPML profiles (fd_cpml.cu:59-192), lam/mu/rho on the padded grid, Ricker
sources (fd_seismogram.cu:166-185) and receivers moved onto the padded grid
(fd_seismogram.cu:153-163), and the FWI window (fd_fwi.cu:28-51).

Synthetic earth models for the five benchmark workloads are built here from
seeded generators (no external data):
  config1  200x200, order 4, homogeneous + circular anomaly, 1 shot, 50 receivers
  config2  800x400, order 8, 6 layers + smoothed +-3% perturbation, 200 receivers
  config3  1000x500, order 8, layers with a dipping fault, 64 shots x 250 receivers
  config4  32 uneven layered models with an elliptical anomaly each
  config5  2000x600, order 8, folded/faulted 30-layer model with wedge and salt body
"""
from __future__ import annotations

from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np

from . import _capi

# Setup helpers (padding, Holberg table, CPML profile, Ricker wavelet, staggered
# averages).  The default is the engine library's host code; any object with the
# same five functions (total_grid, holberg, cpml_profile, wavelet,
# average_parameters) can stand in, e.g. to build a problem in a process that
# must not load the engine library.
_setup = None


def use_setup_helpers(helpers) -> None:
    """Route every later Problem setup through `helpers` (None: the engine library)."""
    global _setup
    _setup = helpers


def _h():
    return _setup if _setup is not None else _capi


@dataclass
class Problem:
    nx: int
    nz: int
    nt: int
    dx: float
    dz: float
    dt: float
    fdorder: int
    npml: int
    fsurf: int = 0
    max_rel_err: int = 1
    # CPML ([PML_boundary], fd_cpml.cu:40-47)
    fpml: float = 10.0
    npower: float = 2.0
    k_max_pml: float = 1.0
    rcoef: float = 1e-3
    damp_v_pml: float = 3000.0
    # derived
    fpad: int = 0
    ppad: int = 0
    nxt: int = 0
    nzt: int = 0
    hc: np.ndarray = field(default_factory=lambda: np.zeros(7))
    cpml: dict = field(default_factory=dict)
    # materials on the padded grid [nzt][nxt]
    lam: Optional[np.ndarray] = None
    mu: Optional[np.ndarray] = None
    rho: Optional[np.ndarray] = None
    # acquisition (padded indices)
    src_x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    src_z: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    src_comp: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    src_shot: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    src_signal: np.ndarray = field(default_factory=lambda: np.zeros((0, 0)))
    rec_x: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    rec_z: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    rec_comp: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    rec_shot: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    nshots: int = 1
    # FWI window (padded, [x1, x2) x [z1, z2))
    fwi_dt: int = 1
    fwi_dx: int = 1
    fwi_dz: int = 1
    x1: int = 0
    x2: int = 0
    z1: int = 0
    z2: int = 0
    name: str = ""

    def finalize(self) -> "Problem":
        self.fpad, self.ppad, self.nxt, self.nzt = _h().total_grid(
            self.nx, self.nz, self.fdorder, self.npml, self.fsurf)
        self.hc = _h().holberg(self.fdorder, self.max_rel_err)
        if self.npml > 0:
            self.cpml = _h().cpml_profile(self.npml, self.dx, self.fpml, self.npower,
                                           self.k_max_pml, self.rcoef, self.damp_v_pml, self.dt)
        else:
            self.cpml = {k: np.zeros(2) for k in ("a", "b", "K", "a_half", "b_half", "K_half")}
        if self.x2 == 0:
            self.x1, self.x2 = 0, self.nxt
        if self.z2 == 0:
            # rows above a free surface hold mirrored stresses only; the window
            # starts at the surface row there (as the reference's default does)
            self.z1, self.z2 = (self.fpad if self.fsurf else 0), self.nzt
        return self

    # --- derived quantities -------------------------------------------------
    @property
    def nft(self) -> int:
        return 1 + (self.nt - 1) // self.fwi_dt

    @property
    def nfz(self) -> int:
        return 1 + (self.z2 - self.z1) // self.fwi_dz

    @property
    def nfx(self) -> int:
        return 1 + (self.x2 - self.x1) // self.fwi_dx

    @property
    def nsrc(self) -> int:
        return len(self.src_x)

    @property
    def nrec(self) -> int:
        return len(self.rec_x)

    def averaged(self):
        """mu_zx, rho_zp, rho_xp (fd_medium.cu:128-159) of the current lam/mu/rho."""
        return _h().average_parameters(self.mu, self.rho)

    def zoff(self) -> int:
        """z offset from the physical grid to the padded one (fd_seismogram.cu:157-160)."""
        return self.fpad if self.fsurf else self.ppad

    def pad_model(self, vp: np.ndarray, vs: np.ndarray, rho: np.ndarray) -> None:
        """Set lam/mu/rho on the padded grid from [nz][nx] velocity/density
        (fd_medium.cu:54-59 conversion), extending edge values into the padding."""
        z0 = self.zoff()
        pads = ((z0, self.nzt - self.nz - z0), (self.ppad, self.nxt - self.nx - self.ppad))
        vp = np.pad(np.asarray(vp, np.float64), pads, mode="edge")
        vs = np.pad(np.asarray(vs, np.float64), pads, mode="edge")
        rho = np.pad(np.asarray(rho, np.float64), pads, mode="edge")
        self.mu = np.ascontiguousarray(vs * vs * rho)
        self.lam = np.ascontiguousarray(vp * vp * rho - 2.0 * self.mu)
        self.rho = np.ascontiguousarray(rho)

    def set_sources(self, x, z, shot, f0, amp=1.0, ts=0.0, comp=2) -> None:
        x = np.asarray(x, np.int32)
        n = len(x)
        self.src_x = (x + self.ppad).astype(np.int32)
        self.src_z = (np.asarray(z, np.int32) + self.zoff()).astype(np.int32)
        self.src_comp = np.full(n, comp, np.int32)
        self.src_shot = np.asarray(shot, np.int32)
        f0 = np.broadcast_to(np.asarray(f0, np.float64), (n,))
        self.src_signal = np.stack([_h().wavelet(self.nt, self.dt, amp, float(f), ts, 1) for f in f0]) \
            if n else np.zeros((0, self.nt))
        self.src_signal = np.ascontiguousarray(self.src_signal)
        self.nshots = int(self.src_shot.max()) + 1 if n else 1

    def set_receivers(self, x, z, shot) -> None:
        x = np.asarray(x, np.int32)
        self.rec_x = (x + self.ppad).astype(np.int32)
        self.rec_z = (np.asarray(z, np.int32) + self.zoff()).astype(np.int32)
        self.rec_comp = np.full(len(x), 2, np.int32)
        self.rec_shot = np.asarray(shot, np.int32)

    def with_model(self, lam, mu, rho) -> "Problem":
        return replace(self, lam=np.ascontiguousarray(lam), mu=np.ascontiguousarray(mu),
                       rho=np.ascontiguousarray(rho))

    def cells(self) -> int:
        return self.nxt * self.nzt


# ---------------------------------------------------------------------------
# earth-model generators
# ---------------------------------------------------------------------------

def gardner(vp):
    return 310.0 * np.asarray(vp, np.float64) ** 0.25


def layered(nz, nx, vps, depths=None):
    """Flat layers with velocities vps from top to bottom (equal thickness)."""
    n = len(vps)
    edges = depths if depths is not None else np.linspace(0, nz, n + 1)[1:-1]
    vp = np.empty((nz, nx))
    zi = np.arange(nz)[:, None]
    layer = np.searchsorted(np.asarray(edges), zi, side="right")
    vp[:] = np.asarray(vps, np.float64)[layer]
    return vp


def smooth_perturbation(shape, sigma_cells, amplitude, seed):
    from scipy.ndimage import gaussian_filter
    rng = np.random.default_rng(seed)
    f = gaussian_filter(rng.standard_normal(shape), sigma_cells, mode="reflect")
    f *= amplitude / np.max(np.abs(f))
    return f


def surface_spread(nx, n, margin=0):
    return np.linspace(margin, nx - 1 - margin, n).round().astype(np.int32)


def config1(anomaly: bool = True) -> Problem:
    """200x200, dx=10, dt=1ms, nt=1000, order 4, npml 20; homogeneous with a
    300 m circle at -10% Vp/Vs (anomaly=True gives the true model)."""
    p = Problem(nx=200, nz=200, nt=1000, dx=10.0, dz=10.0, dt=1e-3, fdorder=4, npml=20,
                fpml=10.0, damp_v_pml=3000.0, name="config1").finalize()
    vp = np.full((200, 200), 3000.0)
    vs = np.full((200, 200), 1732.0)
    if anomaly:
        zz, xx = np.mgrid[0:200, 0:200]
        inside = (zz - 100) ** 2 + (xx - 100) ** 2 <= 30 ** 2
        vp[inside] *= 0.9
        vs[inside] *= 0.9
    p.pad_model(vp, vs, np.full((200, 200), 2000.0))
    p.set_sources([100], [10], [0], 10.0)
    p.set_receivers(np.arange(0, 200, 4), np.full(50, 10), np.zeros(50, np.int32))
    return p


def config2(perturbed: bool = True, nx: int = 800, nz: int = 400, nt: int = 4000, npml: int = 30,
            nrec: int = 200, seed: int = 2) -> Problem:
    """800x400, dx=5, dt=0.5ms, nt=4000, order 8, npml 30; 6 flat layers
    1800->4500 m/s, Vs=Vp/1.73, Gardner density, +-3% smoothed perturbation
    (correlation length 100 m).  The size arguments give the same physics on a
    smaller grid or a shorter record."""
    p = Problem(nx=nx, nz=nz, nt=nt, dx=5.0, dz=5.0, dt=0.5e-3, fdorder=8, npml=npml,
                fpml=15.0, damp_v_pml=4500.0, name="config2").finalize()
    vp = layered(nz, nx, np.linspace(1800.0, 4500.0, 6))
    if perturbed:
        vp = vp * (1.0 + smooth_perturbation((nz, nx), 100.0 / 5.0, 0.03, seed=seed))
    p.pad_model(vp, vp / 1.73, gardner(vp))
    p.set_sources([nx // 2], [5], [0], 15.0)
    p.set_receivers(surface_spread(nx, nrec), np.full(nrec, 5), np.zeros(nrec, np.int32))
    return p


def config3(faulted: bool = True, nshots: int = 64, nrec: int = 250) -> Problem:
    """1000x500, dx=10, dt=1ms, nt=3000, order 8, npml 30; the config2 layering
    with a dipping fault of 200 m throw; nshots at z=5, nrec receivers per shot."""
    nx, nz = 1000, 500
    p = Problem(nx=nx, nz=nz, nt=3000, dx=10.0, dz=10.0, dt=1e-3, fdorder=8, npml=30,
                fpml=10.0, damp_v_pml=4500.0, name="config3").finalize()
    vps = np.linspace(1800.0, 4500.0, 6)
    edges = np.linspace(0, nz, 7)[1:-1]
    zi = np.arange(nz)[:, None].astype(np.float64)
    xi = np.arange(nx)[None, :].astype(np.float64)
    # fault plane dipping 60 degrees through x=nx/2 at the surface; hanging wall down-thrown
    hanging = xi > nx / 2 + zi / np.tan(np.radians(60.0))
    shift = np.where(hanging, 200.0 / 10.0, 0.0) if faulted else 0.0
    layer = np.searchsorted(edges, zi - shift, side="right")
    vp = vps[np.clip(layer, 0, len(vps) - 1)]
    vp = np.broadcast_to(vp, (nz, nx)).copy()
    p.pad_model(vp, vp / 1.73, gardner(vp))
    sx = surface_spread(nx, nshots, margin=10)
    p.set_sources(sx, np.full(nshots, 5), np.arange(nshots), 10.0)
    rx = surface_spread(nx, nrec)
    p.set_receivers(np.tile(rx, nshots), np.full(nshots * nrec, 5),
                    np.repeat(np.arange(nshots, dtype=np.int32), nrec))
    return p


def config4_specs(n=32, seed=4):
    rng = np.random.default_rng(seed)
    specs = []
    for i in range(n):
        specs.append(dict(
            nx=int(rng.integers(200, 1201)), nz=int(rng.integers(200, 601)),
            nt=int(rng.integers(1000, 4001)), fdorder=int(rng.choice([4, 8])),
            nlayers=int(rng.integers(3, 11)), f0=float(rng.uniform(5.0, 20.0)),
            vs_ratio=float(rng.uniform(0.45, 0.6)), seed=int(rng.integers(1 << 30))))
    return specs


def config4_model(spec, true_model=True) -> Problem:
    """One uneven-batch member: random layers 1500-5000 m/s, Vs/Vp in
    [0.45, 0.6], Gardner density, one random elliptical anomaly; dx=10 m,
    dt=0.8 ms, npml 30."""
    rng = np.random.default_rng(spec["seed"])
    nx, nz = spec["nx"], spec["nz"]
    p = Problem(nx=nx, nz=nz, nt=spec["nt"], dx=10.0, dz=10.0, dt=0.8e-3,
                fdorder=spec["fdorder"], npml=30, fpml=spec["f0"], damp_v_pml=5000.0,
                name="config4").finalize()
    vps = np.sort(rng.uniform(1500.0, 5000.0, spec["nlayers"]))
    vp = layered(nz, nx, vps)
    if true_model:
        zz, xx = np.mgrid[0:nz, 0:nx]
        cz, cx = rng.uniform(0.3, 0.7) * nz, rng.uniform(0.3, 0.7) * nx
        az, ax = rng.uniform(0.05, 0.15) * nz, rng.uniform(0.05, 0.15) * nx
        inside = ((zz - cz) / az) ** 2 + ((xx - cx) / ax) ** 2 <= 1.0
        vp = np.where(inside, vp * 1.1, vp)
    vs = vp * spec["vs_ratio"]
    p.pad_model(vp, vs, gardner(vp))
    p.set_sources([nx // 2], [5], [0], spec["f0"])
    nr = max(2, nx // 4)
    p.set_receivers(surface_spread(nx, nr), np.full(nr, 5), np.zeros(nr, np.int32))
    return p


def config5(true_model: bool = True, nshots: int = 96, nrec: int = 400) -> Problem:
    """2000x600, dx=7.5, dt=0.6 ms, nt=5000, order 8, npml 40; 30 folded and
    faulted layers 1500-5500 m/s with a seeded wedge and a 4500 m/s salt body;
    the starting model is the true model smoothed with sigma = 300 m."""
    from scipy.ndimage import gaussian_filter
    nx, nz = 2000, 600
    p = Problem(nx=nx, nz=nz, nt=5000, dx=7.5, dz=7.5, dt=0.6e-3, fdorder=8, npml=40,
                fpml=8.0, damp_v_pml=5500.0, name="config5").finalize()
    rng = np.random.default_rng(5)
    zi = np.arange(nz)[:, None].astype(np.float64)
    xi = np.arange(nx)[None, :].astype(np.float64)
    fold = 25.0 * np.sin(2 * np.pi * xi / 900.0) + 10.0 * np.sin(2 * np.pi * xi / 370.0 + 1.0)
    fault = np.where(xi > 1200 + 0.5 * zi, 18.0, 0.0)
    depth = zi - fold - fault
    edges = np.linspace(0, nz, 31)[1:-1]
    vps = np.linspace(1500.0, 5500.0, 30) + rng.normal(0.0, 60.0, 30)
    vp = vps[np.clip(np.searchsorted(edges, depth, side="right"), 0, 29)]
    wx0 = rng.uniform(200, 500)
    wedge = (xi > wx0) & (xi < wx0 + 500) & (zi > 150 + 0.2 * (xi - wx0)) & (zi < 260)
    vp = np.where(wedge, 2600.0, vp)
    salt = ((xi - 1500.0) / 220.0) ** 2 + ((zi - 330.0) / 90.0) ** 2 <= 1.0
    vp = np.where(salt, 4500.0, vp)
    if not true_model:
        vp = gaussian_filter(vp, 300.0 / 7.5, mode="nearest")
    p.pad_model(vp, vp / 1.8, gardner(vp))
    p.set_sources(surface_spread(nx, nshots, margin=20), np.full(nshots, 4), np.arange(nshots), 8.0)
    rx = surface_spread(nx, nrec)
    p.set_receivers(np.tile(rx, nshots), np.full(nshots * nrec, 4),
                    np.repeat(np.arange(nshots, dtype=np.int32), nrec))
    return p


def small(fdorder=4, nx=48, nz=40, nt=120, npml=8, fsurf=0, nshots=1, nrec=6, seed=0,
          perturb=0.0, fwi=(1, 1, 1)) -> Problem:
    """A small heterogeneous problem the CPU oracle finishes in well under a second."""
    rng = np.random.default_rng(seed)
    p = Problem(nx=nx, nz=nz, nt=nt, dx=10.0, dz=10.0, dt=1e-3, fdorder=fdorder, npml=npml,
                fsurf=fsurf, fpml=12.0, damp_v_pml=3500.0, name="small",
                fwi_dt=fwi[0], fwi_dx=fwi[1], fwi_dz=fwi[2]).finalize()
    vp = layered(nz, nx, [2200.0, 2800.0, 3300.0])
    if perturb:
        vp = vp * (1.0 + perturb * rng.uniform(-1.0, 1.0, vp.shape))
    p.pad_model(vp, vp / 1.8, gardner(vp))
    sx = surface_spread(nx, nshots, margin=4)
    p.set_sources(sx, np.full(nshots, 3), np.arange(nshots), 15.0, amp=1.0)
    rx = surface_spread(nx, nrec, margin=2)
    p.set_receivers(np.tile(rx, nshots), np.full(nshots * nrec, 3),
                    np.repeat(np.arange(nshots, dtype=np.int32), nrec))
    return p
