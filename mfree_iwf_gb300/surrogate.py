"""Learned screen for ring-impact parameter sweeps.

An ensemble of small MLPs (the library's BF16 tensor-core kernels, ``mf_mlp_*``) maps
the parameters of a two-ring impact -- Young's modulus E, Poisson's ratio nu, density
rho, impact speed v, inner and outer radius -- to what the solver reports for it: the
rebound velocity (mean vx of the left ring after the impact), the peak von Mises
stress and a 64-sample contact-force history.  It is trained only on instances the
batched solver itself simulates (:func:`simulate`), and :meth:`Surrogate.screen`
answers a sweep from the network wherever the members agree, handing the rest to the
solver.  No counterpart in the reference.

An instance is the reference's two-body ring impact (rings_monaghan_contact,
rings.cpp:522-621: Gray-Monaghan SPH, penalty contact between the rings' hulls) with
the ring workload's constants (h = 1.3 dx, dt = 0.3 h / c0, alpha = beta = 1,
eta = 0.1, artificial-stress eps 0.3 with exponent 4, XSPH eps 0.5) and a lattice
scaled with the ring: dx = r_out / 20, centres at -+(r_out + dx / 2), which leaves
three dx between the rings' nearest particles (the lattice keeps r < r_out).  The
setup is then self-similar, so the dimensionless outputs depend on r_in / r_out, nu
and v / c0 only; the network is not told this and sees the six raw parameters.
"""
from __future__ import annotations

import ctypes
import math
import re
import time
from dataclasses import dataclass, field
from typing import Dict, Optional, Sequence, Tuple

import numpy as np

from . import METHOD_UL, Simulation, from_scenario, load_library
from . import scenarios as S

PARAM_NAMES = ("E", "nu", "rho", "v", "r_in", "r_out")
# sampling ranges; r_in is drawn as a fraction q of r_out.  They keep v / c0 within
# [0.009, 0.078]: beyond ~0.08 the rings break up in the impact and the rebound stops
# being a regular function of the parameters.
RANGES: Dict[str, Tuple[float, float]] = {
    "E": (3e7, 6e7),
    "nu": (0.3, 0.45),
    "rho": (1000.0, 1500.0),
    "v": (4.0, 10.0),
    "q": (0.6, 0.8),
    "r_out": (0.03, 0.05),
}
N_HISTORY = 64
N_OUT = 2 + N_HISTORY
NR = 20                 # lattice points per outer radius
STEPS = 64 * 50         # solver steps per instance (3200; covers separation over the ranges)
EDGE_TOL = 1e-9         # lattice points this close (relative) to a ring's circles are left out


# ---------------------------------------------------------------- instances
def sample_params(n: int, seed: int) -> np.ndarray:
    """n parameter rows (E, nu, rho, v, r_in, r_out), uniform over the ranges, seeded (PCG64)."""
    rng = np.random.default_rng(seed)
    u = lambda k: rng.uniform(*RANGES[k], size=n)
    E, nu, rho, v, q, ro = u("E"), u("nu"), u("rho"), u("v"), u("q"), u("r_out")
    return np.stack([E, nu, rho, v, q * ro, ro], axis=1)


def impact_instance(p: Sequence[float]) -> S.Scenario:
    """The two-ring impact of one parameter row."""
    E, nu, rho, v, ri, ro = (float(a) for a in p)
    dx = ro / NR
    return S.rings(2 * NR + 1, ro=ro, ri=ri, spacing=ro + 0.5 * dx, rho0=rho, E=E, nu=nu, hdx=1.3, speed=v, dt=None,
                   cfl=0.3, two_bodies=True, alpha=1.0, beta=1.0, eta=0.1, art_stress_eps=0.3, stress_exponent=4.0,
                   xsph_eps=0.5, nbh_eps=S.workload_nbh_eps(dx), edge_tol=EDGE_TOL, exact_hull=True,
                   name="impact instance")


def wave_speed(p: np.ndarray) -> np.ndarray:
    """Bulk wave speed c0 = sqrt(K / rho), K = E / (3 (1 - 2 nu)) (simulation_data.cpp:32-47)."""
    E, nu, rho = p[:, 0], p[:, 1], p[:, 2]
    return np.sqrt(E / (3.0 * (1.0 - 2.0 * nu)) / rho)


def batch_scenario(params: np.ndarray) -> Tuple[S.Scenario, list]:
    """All instances of `params` as one scenario: bodies 2k and 2k+1 are instance k's rings,
    in contact group k, each with its own constants and time step."""
    bodies, groups, first = [], [], None
    for k, p in enumerate(params):
        sc = impact_instance(p)
        for b in sc.bodies:
            b.params = {"E": sc.E, "nu": sc.nu, "rho0": sc.rho0, "dt": sc.dt, "wdeltap": sc.wdeltap}
            bodies.append(b)
            groups.append(k)
        first = first or sc
    ens = S.Scenario(method=METHOD_UL, bodies=bodies, actions=list(first.actions), dt=first.dt, nu=first.nu,
                     E=first.E, rho0=first.rho0, wdeltap=first.wdeltap, corr_exp=first.corr_exp,
                     mghn_eps=first.mghn_eps, alpha=first.alpha, beta=first.beta, eta=first.eta,
                     xsph_eps=first.xsph_eps, nbh_eps=first.nbh_eps, contact=1,
                     name=f"{len(params)} ring impacts")
    return ens, groups


@dataclass
class SolverRun:
    targets: np.ndarray      # [n, N_OUT] physical: rebound (m/s), peak von Mises (Pa), force history (N/m)
    energy_ratio: np.ndarray  # [n] final / initial kinetic energy of the pair (from the rings' mean velocities)
    failed: np.ndarray       # [n] bool: the state went non-finite (targets are NaN)
    particles: int
    seconds: float           # solver wall time, retries included (setup excluded)
    setup_seconds: float
    failures: list = field(default_factory=list)  # (instance, solver message) per failed instance

    @property
    def valid(self) -> np.ndarray:
        """Instances whose solution is physical: finite, the left ring moving back, and no
        kinetic energy gained (the penalty contact can inject energy when the rings
        interpenetrate; those runs are not a response of the material)."""
        return ~self.failed & (self.targets[:, 0] < 0) & (self.energy_ratio <= 1.0)

    @property
    def instances_per_hour(self) -> float:
        return len(self.targets) / self.seconds * 3600.0


def targets_from_monitor(mon: np.ndarray, n: int) -> np.ndarray:
    """[steps, 2n, 4] monitor rows -> [n, N_OUT]: the left ring's mean vx at the last step,
    the peak von Mises stress over both rings and all steps, and the left ring's total
    contact force averaged over N_HISTORY equal windows of steps."""
    steps = mon.shape[0]
    w = steps // N_HISTORY
    out = np.zeros((n, N_OUT), np.float64)
    left = mon[:, 0::2, :]
    right = mon[:, 1::2, :]
    out[:, 0] = left[-1, :, 0]
    out[:, 1] = np.maximum(left[:, :, 2].max(axis=0), right[:, :, 2].max(axis=0))
    fc = left[: w * N_HISTORY, :, 3].reshape(N_HISTORY, w, n).mean(axis=1)
    out[:, 2:] = fc.T
    return out


# the solver names the particle that raised a non-finite state or left its cell grid
_ROW = re.compile(r"MF_ERR_(?:NONFINITE|GRID): .* row (\d+)")


def simulate(params: np.ndarray, precision: str = "mixed", device: int = 0, steps: int = STEPS,
             chunk: int = 2048, check_every: int = 400) -> SolverRun:
    """Run every instance through the batched solver, `chunk` instances per context.

    The solver stops a batch when a state goes non-finite or a particle outruns its cell
    grid, and names the particle; the instance that owns it is marked failed and the
    batch is run again without it."""
    from . import MfError

    params = np.asarray(params, np.float64)
    n = len(params)
    targets = np.full((n, N_OUT), np.nan)
    energy = np.full(n, np.nan)
    failed = np.zeros(n, bool)
    secs, setup, npart, failures = 0.0, 0.0, 0, []
    for c0 in range(0, n, chunk):
        alive = np.arange(c0, min(n, c0 + chunk))
        while len(alive):
            t0 = time.perf_counter()
            ens, groups = batch_scenario(params[alive])
            offsets = np.cumsum([0] + [b.n for b in ens.bodies])
            sim = from_scenario(ens, precision=precision, device=device, groups=groups, graph=True)
            t1 = time.perf_counter()
            try:
                sim.set_monitor(steps)
                done = 0
                while done < steps:
                    k = min(check_every, steps - done)
                    sim.step(k)  # checks the device status after the k steps
                    done += k
                mon = sim.monitor()
            except MfError as e:
                m = _ROW.search(str(e))
                sim.close()
                secs += time.perf_counter() - t1
                setup += t1 - t0
                if m is None:
                    raise
                body = int(np.searchsorted(offsets, int(m.group(1)), side="right")) - 1
                failed[alive[body // 2]] = True
                failures.append((int(alive[body // 2]), str(e)))
                alive = np.delete(alive, body // 2)
                continue
            sim.close()
            t2 = time.perf_counter()
            setup += t1 - t0
            secs += t2 - t1
            npart += ens.n_total
            targets[alive] = targets_from_monitor(mon, len(alive))
            v = params[alive, 3]
            energy[alive] = (mon[-1, 0::2, 0] ** 2 + mon[-1, 0::2, 1] ** 2 + mon[-1, 1::2, 0] ** 2
                             + mon[-1, 1::2, 1] ** 2) / (2.0 * v * v)
            break
    return SolverRun(targets, energy, failed, npart, secs, setup, failures)


# ---------------------------------------------------------------- scaling
def _shells() -> Tuple[np.ndarray, np.ndarray]:
    """The lattice's shells a^2 + b^2 (|a|, |b| <= NR, in units of dx^2, below the outer
    circle) and how many lattice points lie on each."""
    a = np.arange(-NR, NR + 1)
    s2 = (a[:, None] ** 2 + a[None, :] ** 2).ravel()
    s2 = s2[s2 < NR * NR]
    shells, mult = np.unique(s2, return_counts=True)
    return shells, mult


SHELLS, SHELL_MULT = _shells()


def ring_lattice(q: np.ndarray) -> Dict[str, np.ndarray]:
    """What the lattice makes of an inner radius q r_out: the innermost shell kept (the
    lattice keeps distances >= r_in (1 + EDGE_TOL)), the points on it and on the next
    shell out, and the points of one ring.  Radii between two shells give the same ring."""
    q = np.asarray(q, np.float64)
    k = np.searchsorted(SHELLS, (q * NR) ** 2 * (1.0 + EDGE_TOL) ** 2, side="left")
    tail = np.cumsum(SHELL_MULT[::-1])[::-1]  # points on shells k and beyond
    return {"q": np.sqrt(SHELLS[k]) / NR, "inner": SHELL_MULT[k].astype(np.float64),
            "next": SHELL_MULT[np.minimum(k + 1, len(SHELLS) - 1)].astype(np.float64),
            "points": tail[k].astype(np.float64)}


def _feature_columns(params: np.ndarray) -> list:
    p = np.asarray(params, np.float64)
    lat = ring_lattice(p[:, 4] / p[:, 5])
    return [lat["q"], p[:, 1], np.log(p[:, 3] / wave_speed(p)), lat["inner"], lat["points"], lat["next"]]


def _feature_limits() -> list:
    # bounds over the sampling ranges: the lattice columns over every shell the q range
    # can reach, log(v / c0) at its corners
    lat = ring_lattice(np.linspace(*RANGES["q"], 4001))
    E, nu, rho, v = (np.array(RANGES[k]) for k in ("E", "nu", "rho", "v"))
    corners = np.array(np.meshgrid(E, nu, rho, v)).reshape(4, -1).T
    logm = np.log(corners[:, 3] / wave_speed(corners[:, :3]))
    lims = [(lat["q"].min(), lat["q"].max()), tuple(RANGES["nu"]), (logm.min(), logm.max())]
    lims += [(lat[k].min(), max(lat[k].max(), lat[k].min() + 1.0)) for k in ("inner", "points", "next")]
    return lims


FEATURE_LIMITS = _feature_limits()


def features(params: np.ndarray) -> np.ndarray:
    """Network inputs from (E, nu, rho, v, r_in, r_out), each mapped to about [-1, 1].

    An instance's dimensionless outputs depend on the parameters only through nu, the
    Mach number v / c0 and the ring the lattice makes of r_in / r_out (the setup is
    self-similar in r_out, and E and rho enter through c0 and the stress scale), so the
    network sees: the lattice ring's inner radius / r_out, nu, log(v / c0), the points
    on the ring's innermost and next shells, and the ring's point count.  The rebound
    jumps from one lattice ring to the next; the point counts let the network tell
    neighbouring rings apart."""
    cols = _feature_columns(params)
    f = [2.0 * (c - lo) / (hi - lo) - 1.0 for c, (lo, hi) in zip(cols, FEATURE_LIMITS)]
    return np.stack(f, axis=1).astype(np.float32)


def dimensionless(params: np.ndarray, targets: np.ndarray) -> np.ndarray:
    """Physical targets -> dimensionless: rebound / v, log(peak / (rho c0 v)), force / (rho c0 v r_out)."""
    p = np.asarray(params, np.float64)
    c0 = wave_speed(p)
    rho, v, ro = p[:, 2], p[:, 3], p[:, 5]
    d = np.empty_like(targets, dtype=np.float64)
    d[:, 0] = targets[:, 0] / v
    d[:, 1] = np.log(np.maximum(targets[:, 1], 1e-30) / (rho * c0 * v))
    d[:, 2:] = targets[:, 2:] / (rho * c0 * v * ro)[:, None]
    return d


def physical(params: np.ndarray, d: np.ndarray) -> np.ndarray:
    """Inverse of :func:`dimensionless` (works on [..., n, N_OUT])."""
    p = np.asarray(params, np.float64)
    c0 = wave_speed(p)
    rho, v, ro = p[:, 2], p[:, 3], p[:, 5]
    t = np.empty_like(d, dtype=np.float64)
    t[..., 0] = d[..., 0] * v
    t[..., 1] = np.exp(d[..., 1]) * rho * c0 * v
    t[..., 2:] = d[..., 2:] * (rho * c0 * v * ro)[:, None]
    return t


# ---------------------------------------------------------------- the network
class MlpConfig(ctypes.Structure):
    _fields_ = [("members", ctypes.c_int32), ("n_layers", ctypes.c_int32), ("dims", ctypes.c_int32 * 9),
                ("max_batch", ctypes.c_int32), ("device", ctypes.c_int32), ("seed", ctypes.c_uint64)]


def _mlp_lib():
    lib = load_library()
    if getattr(lib, "_mlp_ready", False):
        return lib
    C = ctypes
    FP = C.POINTER(C.c_float)
    sig = {
        "mf_mlp_create": (C.c_int32, [C.POINTER(MlpConfig), C.POINTER(C.c_void_p)]),
        "mf_mlp_destroy": (None, [C.c_void_p]),
        "mf_mlp_last_error": (C.c_char_p, [C.c_void_p]),
        "mf_mlp_num_params": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
        "mf_mlp_get_params": (C.c_int32, [C.c_void_p, C.c_int32, FP]),
        "mf_mlp_set_params": (C.c_int32, [C.c_void_p, C.c_int32, FP]),
        "mf_mlp_get_grads": (C.c_int32, [C.c_void_p, C.c_int32, FP]),
        "mf_mlp_gradients": (C.c_int32, [C.c_void_p, FP, FP, C.c_int32, FP]),
        "mf_mlp_set_data": (C.c_int32, [C.c_void_p, FP, FP, C.c_int32]),
        "mf_mlp_train": (C.c_int32, [C.c_void_p, C.c_int32, C.c_float, C.c_float, FP]),
        "mf_mlp_predict": (C.c_int32, [C.c_void_p, FP, C.c_int32, FP]),
        "mf_mlp_launch_count": (C.c_int32, [C.c_void_p, C.POINTER(C.c_uint64)]),
        "mf_mlp_get_stream": (C.c_int32, [C.c_void_p, C.POINTER(C.c_void_p)]),
        "mf_mlp_set_option": (C.c_int32, [C.c_void_p, C.c_char_p, C.c_int64]),
        "mf_mlp_get_option": (C.c_int32, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    lib._mlp_ready = True
    return lib


def _fp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Mlp:
    """An ensemble of MLPs on the GPU (ReLU hidden layers, linear output)."""

    def __init__(self, dims: Sequence[int], members: int = 5, max_batch: int = 512, seed: int = 1, device: int = 0):
        from . import MfError

        self._lib = _mlp_lib()
        self._err = MfError
        cfg = MlpConfig()
        cfg.members, cfg.n_layers = members, len(dims) - 1
        for i, d in enumerate(dims):
            cfg.dims[i] = d
        cfg.max_batch, cfg.device, cfg.seed = max_batch, device, seed
        h = ctypes.c_void_p()
        st = self._lib.mf_mlp_create(ctypes.byref(cfg), ctypes.byref(h))
        if st != 0:
            raise MfError(st, "mf_mlp_create")
        self._h = h
        self.dims, self.members, self.max_batch = list(dims), members, max_batch

    def _check(self, st: int, what: str) -> None:
        if st != 0:
            raise self._err(st, f"{what}: {self._lib.mf_mlp_last_error(self._h).decode()}")

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.mf_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def num_params(self) -> int:
        n = ctypes.c_uint64()
        self._check(self._lib.mf_mlp_num_params(self._h, ctypes.byref(n)), "mf_mlp_num_params")
        return n.value

    def get_params(self, member: int) -> np.ndarray:
        out = np.zeros(self.num_params, np.float32)
        self._check(self._lib.mf_mlp_get_params(self._h, member, _fp(out)), "mf_mlp_get_params")
        return out

    def set_params(self, member: int, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == self.num_params
        self._check(self._lib.mf_mlp_set_params(self._h, member, _fp(p)), "mf_mlp_set_params")

    def gradients(self, x: np.ndarray, y: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        """x [members, batch, in], y [members, batch, out] -> (grads [members, P], loss [members])."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        loss = np.zeros(self.members, np.float32)
        self._check(self._lib.mf_mlp_gradients(self._h, _fp(x), _fp(y), x.shape[1], _fp(loss)), "mf_mlp_gradients")
        g = np.zeros((self.members, self.num_params), np.float32)
        for z in range(self.members):
            self._check(self._lib.mf_mlp_get_grads(self._h, z, _fp(g[z])), "mf_mlp_get_grads")
        return g, loss

    def set_data(self, x: np.ndarray, y: np.ndarray) -> None:
        x = np.ascontiguousarray(x, np.float32)
        y = np.ascontiguousarray(y, np.float32)
        self._check(self._lib.mf_mlp_set_data(self._h, _fp(x), _fp(y), len(x)), "mf_mlp_set_data")

    def train(self, steps: int, lr0: float, lr1: float) -> np.ndarray:
        hist = np.zeros((steps, self.members), np.float32)
        self._check(self._lib.mf_mlp_train(self._h, steps, lr0, lr1, _fp(hist)), "mf_mlp_train")
        return hist

    def predict(self, x: np.ndarray) -> np.ndarray:
        """x [n, in] -> [members, n, out]."""
        x = np.ascontiguousarray(x, np.float32)
        y = np.zeros((self.members, len(x), self.dims[-1]), np.float32)
        self._check(self._lib.mf_mlp_predict(self._h, _fp(x), len(x), _fp(y)), "mf_mlp_predict")
        return y

    def launch_count(self) -> int:
        n = ctypes.c_uint64()
        self._check(self._lib.mf_mlp_launch_count(self._h, ctypes.byref(n)), "mf_mlp_launch_count")
        return n.value

    def set_option(self, key: str, value: int) -> None:
        self._check(self._lib.mf_mlp_set_option(self._h, key.encode(), int(value)), f"mf_mlp_set_option({key})")

    def get_option(self, key: str) -> int:
        v = ctypes.c_int64()
        self._check(self._lib.mf_mlp_get_option(self._h, key.encode(), ctypes.byref(v)), f"mf_mlp_get_option({key})")
        return v.value


# ---------------------------------------------------------------- the screen
@dataclass
class Screened:
    targets: np.ndarray       # [n, N_OUT] physical outputs (network where accepted, solver elsewhere)
    accepted: np.ndarray      # [n] bool: answered by the network
    disagreement: np.ndarray  # [n] relative spread of the members' rebound velocities
    seconds_network: float
    seconds_solver: float


class Surrogate:
    """Five-member 6 -> 256 -> 256 -> 256 -> 66 ensemble with the screening rule."""

    REBOUND_WEIGHT = 10.0  # the rebound column's scale in the loss (weight 100 in the MSE)

    def __init__(self, members: int = 5, hidden: Sequence[int] = (256, 256, 256), max_batch: int = 512,
                 seed: int = 7, device: int = 0):
        self.mlp = Mlp([len(FEATURE_LIMITS), *hidden, N_OUT], members=members, max_batch=max_batch, seed=seed, device=device)
        self.device = device
        self.mu = np.zeros(N_OUT)
        self.sd = np.ones(N_OUT)
        self.threshold = 0.0

    def _encode(self, params: np.ndarray, targets: np.ndarray) -> np.ndarray:
        d = (dimensionless(params, targets) - self.mu) / self.sd
        d[:, 0] *= self.REBOUND_WEIGHT
        return d.astype(np.float32)

    def _decode(self, params: np.ndarray, z: np.ndarray) -> np.ndarray:
        z = np.array(z, np.float64)
        z[..., 0] /= self.REBOUND_WEIGHT
        return physical(params, z * self.sd + self.mu)

    def fit(self, params: np.ndarray, targets: np.ndarray, steps: int = 6000, lr0: float = 2e-3,
            lr1: float = 2e-5) -> np.ndarray:
        d = dimensionless(params, targets)
        self.mu = d.mean(axis=0)
        self.sd = d.std(axis=0) + 1e-12
        self.mlp.set_data(features(params), self._encode(params, targets))
        return self.mlp.train(steps, lr0, lr1)

    def predict_members(self, params: np.ndarray) -> np.ndarray:
        """[members, n, N_OUT] physical outputs of every member."""
        return self._decode(params, self.mlp.predict(features(params)))

    def predict(self, params: np.ndarray) -> Tuple[np.ndarray, np.ndarray]:
        """(ensemble-mean physical outputs [n, N_OUT], rebound disagreement [n])."""
        y = self.predict_members(params)
        mean = y.mean(axis=0)
        spread = y[:, :, 0].std(axis=0) / np.maximum(np.abs(mean[:, 0]), 1e-12)
        return mean, spread

    def calibrate(self, params: np.ndarray, targets: np.ndarray, max_error: float = 0.02,
                  quantile: float = 0.95) -> float:
        """Largest disagreement threshold whose accepted instances keep the `quantile`
        of the rebound error within max_error; returns (and keeps) the threshold."""
        mean, spread = self.predict(params)
        err = np.abs(mean[:, 0] - targets[:, 0]) / np.abs(targets[:, 0])
        order = np.argsort(spread)
        best = 0.0
        for k in range(1, len(order) + 1):
            acc = err[order[:k]]
            if np.quantile(acc, quantile) <= max_error:
                best = float(spread[order[k - 1]])
        self.threshold = best
        return best

    def screen(self, params: np.ndarray, precision: str = "mixed", chunk: int = 2048) -> Screened:
        """Answer every instance from the network when its members agree within the
        threshold, else from the solver."""
        t0 = time.perf_counter()
        mean, spread = self.predict(params)
        t1 = time.perf_counter()
        acc = spread <= self.threshold
        out = mean.copy()
        t_solver = 0.0
        if (~acc).any():
            run = simulate(params[~acc], precision=precision, device=self.device, chunk=chunk)
            out[~acc] = run.targets
            t_solver = run.seconds + run.setup_seconds
        return Screened(out, acc, spread, t1 - t0, t_solver)


# ---------------------------------------------------------------- the sweep experiment
def run_experiment(n_train: int = 20000, n_test: int = 1000, val_frac: float = 0.1, train_steps: int = 20000,
                   seed: int = 20261203, data: Optional[str] = None, device: int = 0) -> dict:
    """Generate a training set with the batched solver, train the ensemble, calibrate the
    disagreement threshold on a held-out slice of it, then screen a fresh sweep and
    compare with the solver alone on that sweep.  `data` (an .npz path) caches the
    solver's training outputs between runs."""
    import os

    train_p = sample_params(n_train, seed)
    test_p = sample_params(n_test, seed + 1)
    gen_seconds = None
    if data and os.path.exists(data):
        z = np.load(data)
        assert np.array_equal(z["params"], train_p), "cached data set was made with other parameters"
        train_t = z["targets"]
    else:
        run = simulate(train_p, device=device)
        train_t, gen_seconds = run.targets.copy(), run.seconds + run.setup_seconds
        train_t[~run.valid] = np.nan
        if data:
            np.savez_compressed(data, params=train_p, targets=train_t)
    ok = np.all(np.isfinite(train_t), axis=1) & (train_t[:, 0] < 0)
    n_fit = int(n_train * (1 - val_frac))
    fit_idx = np.nonzero(ok[:n_fit])[0]
    val_idx = n_fit + np.nonzero(ok[n_fit:])[0]
    sur = Surrogate(device=device)
    t0 = time.perf_counter()
    hist = sur.fit(train_p[fit_idx], train_t[fit_idx], steps=train_steps)
    t_train = time.perf_counter() - t0
    thr = sur.calibrate(train_p[val_idx], train_t[val_idx])
    truth = simulate(test_p, device=device)                # the solver-only sweep
    res = sur.screen(test_p)
    good = truth.valid  # instances whose solver answer is itself physical
    err = np.abs(res.targets[:, 0] - truth.targets[:, 0]) / np.abs(truth.targets[:, 0])
    net_only, _ = sur.predict(test_p)
    err_net = (np.abs(net_only[:, 0] - truth.targets[:, 0]) / np.abs(truth.targets[:, 0]))[good]
    t_solver = truth.seconds + truth.setup_seconds
    t_screen = res.seconds_network + res.seconds_solver
    acc = res.accepted & good
    return {
        "n_train": int(len(fit_idx)), "n_val": int(len(val_idx)), "n_test": n_test,
        "train_invalid": int((~ok).sum()), "test_invalid": int((~good).sum()),
        "generate_seconds": gen_seconds, "train_seconds": t_train, "train_steps": train_steps,
        "final_loss": float(hist[-100:].mean()),
        "threshold": thr, "accepted_fraction": float(res.accepted.mean()),
        "rebound_rel_error_accepted": {"mean": float(err[acc].mean()) if acc.any() else None,
                                       "p95": float(np.quantile(err[acc], 0.95)) if acc.any() else None,
                                       "max": float(err[acc].max()) if acc.any() else None},
        "rebound_rel_error_network_all": {"mean": float(err_net.mean()), "p95": float(np.quantile(err_net, 0.95))},
        "solver_only": {"seconds": t_solver, "instances_per_hour": n_test / t_solver * 3600.0},
        "screened": {"seconds": t_screen, "network_seconds": res.seconds_network,
                     "solver_seconds": res.seconds_solver, "instances_per_hour": n_test / t_screen * 3600.0},
        "gain": t_solver / t_screen,
    }



def gemm_benchmark(rows: int = 65535, chunks: int = 16, members: int = 5, device: int = 0,
                   tcgen05: Optional[int] = None, fused: Optional[int] = None) -> dict:
    """Inference throughput of the ensemble on device-resident inputs and outputs:
    `chunks` x `rows` rows through 6 -> 256 -> 256 -> 256 -> 66, timed with CUDA events
    on the library's stream; FLOPs counted on the true (unpadded) layer sizes.  `tcgen05`
    selects the tensor-core path of the forward products and `fused` the whole-network
    kernel (one launch over every row) against per-layer GEMMs over passes of `rows`
    rows (None: the library's defaults)."""
    import torch

    dims = [len(FEATURE_LIMITS), 256, 256, 256, N_OUT]
    mlp = Mlp(dims, members=members, max_batch=rows, seed=1, device=device)
    if tcgen05 is not None:
        mlp.set_option("tcgen05", tcgen05)
    if fused is not None:
        mlp.set_option("fused", fused)
    n = rows * chunks
    x = torch.rand(n, dims[0], device=f"cuda:{device}", dtype=torch.float32) * 2 - 1
    y = torch.empty(members, n, dims[-1], device=f"cuda:{device}", dtype=torch.float32)
    fp = lambda t: ctypes.cast(t.data_ptr(), ctypes.POINTER(ctypes.c_float))
    lib = mlp._lib
    s = ctypes.c_void_p()
    lib.mf_mlp_get_stream(mlp._h, ctypes.byref(s))
    stream = torch.cuda.ExternalStream(s.value)
    for _ in range(3):  # warm-up
        mlp._check(lib.mf_mlp_predict(mlp._h, fp(x), n, fp(y)), "mf_mlp_predict")
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    reps = 5
    for _ in range(reps):
        mlp._check(lib.mf_mlp_predict(mlp._h, fp(x), n, fp(y)), "mf_mlp_predict")
    e1.record(stream)
    torch.cuda.synchronize()
    secs = e0.elapsed_time(e1) / 1e3 / reps
    flop_row = 2 * sum(dims[i] * dims[i + 1] for i in range(len(dims) - 1))
    flops = flop_row * members * n
    tc, fz = mlp.get_option("tcgen05"), mlp.get_option("fused")
    mlp.close()
    return {"rows_per_pass": rows, "instances": n, "members": members, "seconds": secs,
            "instances_per_s": n / secs, "tflops": flops / secs / 1e12, "flop_per_instance_member": flop_row,
            "tcgen05": tc, "fused": fz}


if __name__ == "__main__":
    import argparse
    import json

    ap = argparse.ArgumentParser(description="surrogate-screened ring-impact sweep against the solver alone")
    ap.add_argument("--train", type=int, default=20000)
    ap.add_argument("--test", type=int, default=1000)
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--data", default=None, help=".npz cache of the training set's solver outputs")
    ap.add_argument("--out", default=None, help="write the JSON result here too")
    ap.add_argument("--gemm-bench", action="store_true", help="only time the ensemble's inference GEMMs")
    ap.add_argument("--tcgen05", type=int, choices=[0, 1], default=None, help="with --gemm-bench: the GEMM path")
    ap.add_argument("--fused", type=int, choices=[0, 1], default=None,
                    help="with --gemm-bench: the whole-network kernel (1) or per-layer GEMMs (0)")
    ap.add_argument("--chunks", type=int, default=16, help="with --gemm-bench: passes of 65,535 rows")
    a = ap.parse_args()
    r = (gemm_benchmark(chunks=a.chunks, tcgen05=a.tcgen05, fused=a.fused) if a.gemm_bench
         else run_experiment(a.train, a.test, train_steps=a.steps, data=a.data))
    s = json.dumps(r, indent=1)
    print(s)
    if a.out:
        with open(a.out, "w") as f:
            f.write(s + "\n")
