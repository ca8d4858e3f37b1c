"""Closure: the learned correction of a 4x-coarsened lattice (lbm_closure_*).

A three-layer 3x3 convolution (9 -> 32 -> 32 -> 9 channels, BF16 weights and activations,
FP32 accumulation on the tensor cores) maps the non-equilibrium part of a coarse cell's
populations to a correction of those populations, projected so that no cell's density or
momentum changes.  It is trained on the GPU (the library's own forward, backward and Adam
kernels) on pairs (coarse state after k coarse steps, coarse-grained fine state k*factor
fine steps later).
"""
import ctypes

import numpy as np

from . import _native as nat


def coarsen(fine, coarse, factor: int, neq_scale: float):
    """Write the coarse-grained state of FluidSimulator `fine` into `coarse`."""
    nat.check(nat.load().lbm_coarsen(fine.handle, coarse.handle, int(factor), float(neq_scale)))


class Closure:
    INPUTS = {"neq": 0, "eq": 1}
    TARGETS = {"populations": 0, "equilibrium": 1, "momentum": 2, "stress": 3}
    PROJECTIONS = {"cell": 0, "domain": 1}

    def __init__(self, nx: int, ny: int, seed: int = 0, s_in: float = 1000.0, s_out: float = 1000.0,
                 inputs: str = "neq", target: str = "populations", projection: str = "cell"):
        lib = nat.load()
        h = ctypes.c_void_p()
        nat.check(lib.lbm_closure_create(int(nx), int(ny), int(seed), ctypes.byref(h)))
        self._lib, self._h = lib, h
        self.nx, self.ny = int(nx), int(ny)
        self.nparams = lib.lbm_closure_param_count()
        self.set_scales(s_in, s_out)
        self.set_form(inputs, target, projection)
        self.crop = None

    def close(self):
        if getattr(self, "_h", None):
            self._lib.lbm_closure_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_scales(self, s_in: float, s_out: float):
        nat.check(self._lib.lbm_closure_set_scales(self._h, float(s_in), float(s_out)))
        self.s_in, self.s_out = float(s_in), float(s_out)

    def set_form(self, inputs: str = "neq", target: str = "populations", projection: str = "cell"):
        """inputs 'neq' (s_in * f_neq) or 'eq' (s_in * (f_eq(rho, u) - w)); target
        'populations' (target - pred) or 'equilibrium' (difference of the equilibrium parts);
        projection 'cell' (no cell's rho or j changes) or 'domain' (the lattice's totals do not)."""
        nat.check(self._lib.lbm_closure_set_form(self._h, self.INPUTS[inputs], self.TARGETS[target],
                                                 self.PROJECTIONS[projection]))
        self.inputs, self.target, self.projection = inputs, target, projection

    def set_stress_factor(self, factor: float):
        """Stress target: window of a pair in coarse steps / (2 x steps between applications)."""
        nat.check(self._lib.lbm_closure_set_stress_factor(self._h, float(factor)))
        self.stress_factor = float(factor)

    KERNELS = {"fused": 0, "layers": 1}

    def set_kernel(self, kernel: str = "fused"):
        """'fused': apply / predict as one tcgen05 kernel with the activations on chip, and the
        training weight gradients on the tcgen05 tensor cores; 'layers': feature kernel + one
        mma.sync kernel per layer, and the weight gradients on the CUDA cores."""
        nat.check(self._lib.lbm_closure_set_kernel(self._h, self.KERNELS[kernel]))
        self.kernel = kernel

    def status(self):
        """Synchronises; raises LbmError if the fused kernel gave up on a bounded wait."""
        nat.check(self._lib.lbm_closure_status(self._h))

    @property
    def params(self) -> np.ndarray:
        out = np.empty(self.nparams, np.float32)
        nat.check(self._lib.lbm_closure_get_params(self._h, nat.ptr(out)))
        return out

    @params.setter
    def params(self, p):
        p = np.ascontiguousarray(p, np.float32)
        assert p.size == self.nparams
        nat.check(self._lib.lbm_closure_set_params(self._h, nat.ptr(p)))

    def apply(self, sim, strength: float = 1.0):
        """Correct the current populations of FluidSimulator `sim` in place; `strength` scales
        the correction (the output scale s_out is divided by it for this call)."""
        if strength == 1.0:
            nat.check(self._lib.lbm_closure_apply(self._h, sim.handle))
            return
        s_in, s_out = self.s_in, self.s_out
        self.set_scales(s_in, s_out / strength)
        try:
            nat.check(self._lib.lbm_closure_apply(self._h, sim.handle))
        finally:
            self.set_scales(s_in, s_out)

    def predict(self, sim) -> np.ndarray:
        """The correction the closure would add to `sim`, shape (9, ny, nx)."""
        out = np.empty((9, self.ny, self.nx), np.float32)
        nat.check(self._lib.lbm_closure_predict(self._h, sim.handle, nat.ptr(out)))
        return out

    def reserve(self, max_pairs: int, crop: int, batch: int):
        nat.check(self._lib.lbm_closure_reserve(self._h, int(max_pairs), int(crop), int(batch)))
        self.crop = int(crop)

    def add_pair(self, pred, target, ox: int, oy: int):
        nat.check(self._lib.lbm_closure_add_pair(self._h, pred.handle, target.handle, int(ox), int(oy)))

    @property
    def npairs(self) -> int:
        n = ctypes.c_int32()
        nat.check(self._lib.lbm_closure_pairs(self._h, ctypes.byref(n)))
        return int(n.value)

    def train(self, iters: int, lr: float = 1e-3, seed: int = 0) -> float:
        loss = ctypes.c_double()
        nat.check(self._lib.lbm_closure_train(self._h, int(iters), float(lr), int(seed), ctypes.byref(loss)))
        return float(loss.value)

    def eval(self, begin: int, end: int) -> float:
        loss = ctypes.c_double()
        nat.check(self._lib.lbm_closure_eval(self._h, int(begin), int(end), ctypes.byref(loss)))
        return float(loss.value)

    def loss_grad(self, feats: np.ndarray, targets: np.ndarray):
        """Mean loss and logical gradient for host crops feats/targets of shape (n, S, S, 9)."""
        feats = np.ascontiguousarray(feats, np.float32)
        targets = np.ascontiguousarray(targets, np.float32)
        n, S = feats.shape[0], feats.shape[1]
        loss = ctypes.c_double()
        g = np.empty(self.nparams, np.float32)
        nat.check(self._lib.lbm_closure_loss_grad(self._h, n, S, nat.ptr(feats), nat.ptr(targets), ctypes.byref(loss),
                                                  nat.ptr(g)))
        return float(loss.value), g


# ---------------------------------------------------------------------------------------
# periodic decaying turbulence: data, training and evaluation of the closure
# ---------------------------------------------------------------------------------------
class TurbulenceSetup:
    """Fine lattice nf x nf with tau_f; coarse lattice nf/factor with the acoustically
    scaled viscosity (tau_c - 1/2 = (tau_f - 1/2) / factor); the closure acts every
    k_coarse coarse steps."""

    def __init__(self, nf=4096, factor=4, tau_f=0.5005, k_coarse=4, k0=8.0, u_rms=0.04, collision="mrt"):
        self.nf, self.factor, self.tau_f, self.k_coarse = nf, factor, tau_f, k_coarse
        self.nc = nf // factor
        self.tau_c = 0.5 + (tau_f - 0.5) / factor
        # f_neq scales with tau times the velocity gradient per cell: x factor on the coarse grid
        self.neq_scale = factor * self.tau_c / tau_f
        self.k0, self.u_rms, self.collision = k0, u_rms, collision

    def fine(self, seed):
        from .fluid import FluidSimulator
        from .turbulence import random_velocity

        s = FluidSimulator(self.nf, self.nf, mode="physics", scene="periodic", tau=self.tau_f,
                           collision=self.collision)
        ux, uy = random_velocity(self.nf, seed, self.k0, self.u_rms)
        s.init_equilibrium(None, ux.astype(np.float32), uy.astype(np.float32))
        return s

    def coarse(self):
        from .fluid import FluidSimulator

        return FluidSimulator(self.nc, self.nc, mode="physics", scene="periodic", tau=self.tau_c,
                              collision=self.collision)


_W9 = np.array([4 / 9] + [1 / 9] * 4 + [1 / 36] * 4)
_EX = np.array([0, 1, 0, -1, 0, 1, -1, -1, 1], dtype=np.float64)
_EY = np.array([0, 0, -1, 0, 1, -1, -1, 1, 1], dtype=np.float64)


def _neq_and_momentum(f):
    """f: (9, ny, nx) absolute populations -> (f_neq, rho, jx, jy)."""
    rho = f.sum(0)
    jx = (f * _EX[:, None, None]).sum(0)
    jy = (f * _EY[:, None, None]).sum(0)
    ux, uy = jx / rho, jy / rho
    eu = _EX[:, None, None] * ux + _EY[:, None, None] * uy
    feq = _W9[:, None, None] * rho * (1 + 3 * eu + 4.5 * eu * eu - 1.5 * (ux * ux + uy * uy))
    return f - feq, rho, jx, jy


def _project(v):
    s = v.sum(0)
    sx = (v * _EX[:, None, None]).sum(0)
    sy = (v * _EY[:, None, None]).sum(0)
    return v - _W9[:, None, None] * (s + 3 * (_EX[:, None, None] * sx + _EY[:, None, None] * sy))


def generate_pairs(closure, setup, seeds, snapshots=125, interval=160, crop=256, rng_seed=0, log=None,
                   sources=("fresh", "rollout"), corrected=None, calibrate=True, window=None):
    """Training pairs from `snapshots` snapshots of every seed, taken every `interval` fine
    steps over one fine run.  Each snapshot adds one pair per source:

    * "fresh": the coarse-grained fine state advanced k_coarse coarse steps;
    * "rollout": a coarse lattice that has run alongside the fine one since the coarse-grained
      initial state -- with the closure `corrected` applied every k_coarse coarse steps when
      given, as in evaluation -- so the pairs cover the states a long coarse run reaches.

    The target is the coarse-grained fine state at the same time.  A pair spans `window`
    coarse steps (default: the closure's interval k_coarse; the stress target learns from
    longer windows, over which its momentum effect accumulates).  With `calibrate`, the
    feature and output scales are set from the first fresh pair (unit RMS)."""
    rng = np.random.default_rng(rng_seed)
    pred, target = setup.coarse(), setup.coarse()
    w = setup.k_coarse if window is None else int(window)
    kf = w * setup.factor
    assert interval % kf == 0 and interval >= kf

    def roll_steps(roll, n):  # n coarse steps, the closure `corrected` every k_coarse of them
        for _ in range(n // setup.k_coarse):
            roll.step(setup.k_coarse)
            if corrected is not None:
                corrected.apply(roll)
    calibrated = not calibrate
    for seed in seeds:
        fine = setup.fine(seed)
        roll = None
        if "rollout" in sources:
            roll = setup.coarse()
            coarsen(fine, roll, setup.factor, setup.neq_scale)
        for s in range(snapshots):
            if "fresh" in sources:
                coarsen(fine, pred, setup.factor, setup.neq_scale)
                pred.step(w)
            if roll is not None:
                roll_steps(roll, w)
            fine.step(kf)
            coarsen(fine, target, setup.factor, setup.neq_scale)
            if not calibrated:
                fp = pred.read_populations(np.float64)
                ft = target.read_populations(np.float64)
                neq = _neq_and_momentum(fp)[0]
                feat = neq if closure.inputs == "neq" else (fp - _W9[:, None, None]) - neq
                if closure.target == "equilibrium":
                    tgt = (ft - _neq_and_momentum(ft)[0]) - (fp - neq)
                elif closure.target in ("momentum", "stress"):
                    dj = ((ft - fp) * _EX[:, None, None]).sum(0), ((ft - fp) * _EY[:, None, None]).sum(0)
                    tgt = 3.0 * _W9[:, None, None] * (_EX[:, None, None] * dj[0] + _EY[:, None, None] * dj[1])
                else:
                    tgt = ft - fp
                if closure.projection == "cell" and closure.target != "stress":
                    tgt = _project(tgt)
                closure.set_scales(1.0 / max(float(feat.std()), 1e-12), 1.0 / max(float(tgt.std()), 1e-12))
                calibrated = True
            ox, oy = int(rng.integers(0, setup.nc)), int(rng.integers(0, setup.nc))
            if "fresh" in sources:
                closure.add_pair(pred, target, ox, oy)
            if roll is not None:
                closure.add_pair(roll, target, ox, oy)
                roll_steps(roll, (interval - kf) // setup.factor)
            fine.step(interval - kf)
        if log:
            log("seed %d: %d pairs" % (seed, closure.npairs))
        fine.close()
        if roll is not None:
            roll.close()
    pred.close()
    target.close()


def coarse_velocity_of(sim_fine, factor):
    """Momentum-weighted block average of the fine velocity field."""
    f = sim_fine.read_populations(np.float64)
    rho = f.sum(0)
    jx = (f * _EX[:, None, None]).sum(0)
    jy = (f * _EY[:, None, None]).sum(0)
    ny, nx = rho.shape
    blk = lambda a: a.reshape(ny // factor, factor, nx // factor, factor).mean(axis=(1, 3))
    r = blk(rho)
    return blk(jx) / r, blk(jy) / r


def _run_name(strength):
    return "closure" if strength == 1.0 else "closure@%g" % strength


def evaluate(closure, setup, seed, fine_steps=20000, check_every=2000, strengths=(1.0,)):
    """Run the fine lattice and coarse lattices without the closure and with it at each
    correction strength, all from the coarse-grained initial state; relative L2 velocity error
    of each against the coarse-grained fine run at every checkpoint (keys err_plain,
    err_closure for strength 1, err_closure@<strength> otherwise)."""
    fine = setup.fine(seed)
    plain = setup.coarse()
    corr = {a: setup.coarse() for a in strengths}
    for s in [plain] + list(corr.values()):
        coarsen(fine, s, setup.factor, setup.neq_scale)
    rows = []
    cs = check_every // setup.factor
    assert cs % setup.k_coarse == 0
    for t in range(check_every, fine_steps + 1, check_every):
        fine.step(check_every)
        plain.step(cs)
        for a, s in corr.items():
            for _ in range(cs // setup.k_coarse):
                s.step(setup.k_coarse)
                closure.apply(s, a)
        gx, gy = coarse_velocity_of(fine, setup.factor)
        norm = np.sqrt(np.sum(gx * gx + gy * gy))
        row = {"fine_step": t, "fine_nonfinite": fine.nonfinite_count(), "ke_fine": float(0.5 * np.mean(gx * gx + gy * gy))}
        for name, s in [("plain", plain)] + [(_run_name(a), s) for a, s in corr.items()]:
            _, ux, uy = s.read_macro()
            row["err_" + name] = float(np.sqrt(np.sum((ux - gx) ** 2 + (uy - gy) ** 2)) / norm)
            row["ke_" + name] = float(0.5 * np.mean(ux.astype(np.float64) ** 2 + uy.astype(np.float64) ** 2))
        rows.append(row)
    for s in [fine, plain] + list(corr.values()):
        s.close()
    return rows


def _kinetic_energy(sim):
    _, ux, uy = sim.read_macro()
    return float(0.5 * np.mean(ux.astype(np.float64) ** 2 + uy.astype(np.float64) ** 2))


def advance(closure, setup, seed, fine_steps=20000, check_every=2000, strength=1.0, energy_tol=0.02):
    """Advance the decaying-turbulence case `seed` by fine_steps fine-equivalent steps on the
    coarse lattice corrected by the closure, with the plain fine lattice as the fallback.

    Every check_every fine-equivalent steps the coarse state must be finite and its kinetic
    energy must not have grown by more than energy_tol (relative) since the previous check:
    decaying turbulence only loses energy, so growth marks a correction that feeds the flow.  On a
    failed check the coarse run is abandoned and the fine lattice, kept at the initial state, runs
    the whole span instead.  Returns a dict: ux, uy (on the coarse grid: the corrected run's macro
    field, or the block-averaged fine velocity after a fallback), fallback (bool), failed_at (the
    fine-equivalent step of the failed check or None), energies (kinetic energy at each check)."""
    fine = setup.fine(seed)
    coarse = setup.coarse()
    coarsen(fine, coarse, setup.factor, setup.neq_scale)
    cs = check_every // setup.factor
    assert cs % setup.k_coarse == 0 and fine_steps % check_every == 0
    energies, failed_at = [], None
    ke_prev = None
    for t in range(check_every, fine_steps + 1, check_every):
        for _ in range(cs // setup.k_coarse):
            coarse.step(setup.k_coarse)
            closure.apply(coarse, strength)
        ke = _kinetic_energy(coarse)
        energies.append(ke)
        bad = coarse.nonfinite_count() > 0 or not np.isfinite(ke)
        if not bad and ke_prev is not None and ke > ke_prev * (1.0 + energy_tol):
            bad = True
        if bad:
            failed_at = t
            break
        ke_prev = ke
    if failed_at is None:
        _, ux, uy = coarse.read_macro()
        out = dict(ux=ux, uy=uy, fallback=False)
    else:
        fine.step(fine_steps)
        gx, gy = coarse_velocity_of(fine, setup.factor)
        out = dict(ux=gx.astype(np.float32), uy=gy.astype(np.float32), fallback=True)
    out.update(failed_at=failed_at, energies=energies)
    fine.close()
    coarse.close()
    return out


def time_runs(closure, setup, seed, fine_steps=20000, strength=1.0):
    """Device time (CUDA events on the lattices' streams, synchronised) of the plain fine
    run, the plain coarse run and the coarse run with the closure, over the same span."""
    import torch

    out = {}
    fine = setup.fine(seed)
    plain, corr = setup.coarse(), setup.coarse()
    coarsen(fine, plain, setup.factor, setup.neq_scale)
    coarsen(fine, corr, setup.factor, setup.neq_scale)
    stream = torch.cuda.Stream()
    for s in (fine, plain, corr):
        s.set_stream(stream.cuda_stream)
    nc = fine_steps // setup.factor

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) * 1e-3

    out["fine_s"] = timed(lambda: fine.step(fine_steps))
    out["coarse_plain_s"] = timed(lambda: plain.step(nc))

    def run_corr():
        for _ in range(nc // setup.k_coarse):
            corr.step(setup.k_coarse)
            closure.apply(corr, strength)

    out["coarse_closure_s"] = timed(run_corr)
    out["speedup_closure"] = out["fine_s"] / out["coarse_closure_s"]
    out["speedup_plain"] = out["fine_s"] / out["coarse_plain_s"]
    for s in (fine, plain, corr):
        s.close()
    return out
