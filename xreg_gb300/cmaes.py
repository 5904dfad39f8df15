"""CMA-ES optimizer (libxreg_gb300, xr_cmaes_*) with the call sequence of xReg's
vendored cmaes.c: sample a population, (re)sample out-of-bounds candidates,
update with the objective values, test for termination."""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import call, load

STOP_REASONS = {0: None, 1: "tol_fun", 2: "tol_x", 3: "max_iter", 4: "numerical"}


class CMAES:
    def __init__(self, xstart, stddevs, lam: int, seed: int = 0):
        load()
        x0 = np.ascontiguousarray(xstart, dtype=np.float64)
        sd = np.ascontiguousarray(stddevs, dtype=np.float64)
        assert x0.shape == sd.shape and x0.ndim == 1
        h = C.c_void_p()
        call("xr_cmaes_create", int(x0.size), x0.ctypes.data_as(C.c_void_p), sd.ctypes.data_as(C.c_void_p), int(lam),
             C.c_uint64(int(seed) & 0xFFFFFFFFFFFFFFFF), C.byref(h))
        self._h = h
        self.n = int(x0.size)
        self.lam = int(lam)
        self._pop = np.zeros((self.lam, self.n))
        self.on_device = False

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().xr_cmaes_destroy(h)
            self._h = None

    def set_stop(self, tol_fun: float = 1e-12, tol_x: float = 1e-11, max_iter: int = 1_000_000) -> None:
        call("xr_cmaes_set_stop", self._h, float(tol_fun), float(tol_x), int(max_iter))

    def sample_population(self) -> np.ndarray:
        call("xr_cmaes_sample_population", self._h, self._pop.ctypes.data_as(C.c_void_p))
        return self._pop

    def resample_single(self, k: int) -> np.ndarray:
        call("xr_cmaes_resample_single", self._h, int(k), self._pop.ctypes.data_as(C.c_void_p))
        return self._pop[k]

    def sample_within_bounds(self, bounds) -> np.ndarray:
        """Samples, then redraws every candidate outside [-b, b] until it is inside
        (Intensity2D3DRegiCMAES::run, xregIntensity2D3DRegiCMAES.cpp:162-191)."""
        pop = self.sample_population()
        if bounds is None:
            return pop
        b = np.asarray(bounds, dtype=np.float64)
        for k in range(self.lam):
            tries = 0
            while np.any((b > 0.0) & (np.abs(pop[k]) > b)):  # a bound of 0 leaves its coordinate free
                self.resample_single(k)
                tries += 1
                if tries > 100000:
                    raise RuntimeError("CMA-ES: could not sample a candidate inside the bounds")
        return pop

    def update_distribution(self, fvals) -> None:
        f = np.ascontiguousarray(fvals, dtype=np.float64)
        assert f.size == self.lam
        call("xr_cmaes_update_distribution", self._h, f.ctypes.data_as(C.c_void_p))

    def test_for_termination(self):
        r = C.c_int32()
        call("xr_cmaes_test_termination", self._h, C.byref(r))
        return STOP_REASONS.get(r.value, "unknown")

    def attach_device(self, device: int = -1) -> None:
        """Moves the state to device memory: the job-set step
        (api.JobSet.regi_step) then draws and updates it inside its own
        launches, with the same bits as the host methods (which refuse while
        attached; state() and test_for_termination() read the device copy)."""
        call("xr_cmaes_attach_device", self._h, int(device))
        self.on_device = True

    def detach_device(self) -> None:
        """Brings the state back to host memory."""
        call("xr_cmaes_detach_device", self._h)
        self.on_device = False

    def export_state(self) -> bytes:
        """The whole state block (parameters, distribution, last population)."""
        nb = C.c_int64()
        call("xr_cmaes_state_bytes", self._h, C.byref(nb))
        buf = (C.c_ubyte * nb.value)()
        call("xr_cmaes_export_state", self._h, C.cast(buf, C.c_void_p), nb.value)
        return bytes(buf)

    def state(self) -> dict:
        mean = np.zeros(self.n)
        best = np.zeros(self.n)
        bf, sg, gen = C.c_double(), C.c_double(), C.c_int64()
        call("xr_cmaes_get", self._h, mean.ctypes.data_as(C.c_void_p), best.ctypes.data_as(C.c_void_p), C.byref(bf),
             C.byref(sg), C.byref(gen))
        return {"mean": mean, "best_x": best, "best_f": bf.value, "sigma": sg.value, "generation": gen.value}


class TrustRegionDFO:
    """Bound-constrained derivative-free trust-region optimizer (xr_dfo_*,
    Powell's BOBYQA method), the final-level optimizer in place of xReg's NLopt
    LN_BOBYQA: the first ask is the 2n+1 initial points, each later one the
    trust-region or geometry point (or `batch` points, set_batch)."""

    def __init__(self, x0, lower, upper, rho_beg: float, rho_end: float, max_iter: int, batch: int = 1):
        load()
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        lo = np.ascontiguousarray(lower, dtype=np.float64)
        hi = np.ascontiguousarray(upper, dtype=np.float64)
        h = C.c_void_p()
        call("xr_dfo_create", int(x0.size), x0.ctypes.data_as(C.c_void_p), lo.ctypes.data_as(C.c_void_p),
             hi.ctypes.data_as(C.c_void_p), float(rho_beg), float(rho_end), int(max_iter), C.byref(h))
        self._h = h
        self.n = int(x0.size)
        self._buf = np.zeros((2 * self.n + 2, self.n))
        if batch != 1:
            call("xr_dfo_set_batch", self._h, int(batch))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            load().xr_dfo_destroy(h)
            self._h = None

    def ask(self) -> np.ndarray:
        cnt = C.c_int32()
        call("xr_dfo_ask", self._h, self._buf.ctypes.data_as(C.c_void_p), C.byref(cnt))
        return self._buf[:cnt.value].copy()

    def tell(self, fvals) -> None:
        f = np.ascontiguousarray(fvals, dtype=np.float64)
        call("xr_dfo_tell", self._h, f.ctypes.data_as(C.c_void_p))

    def test_for_termination(self):
        r = C.c_int32()
        call("xr_dfo_test_termination", self._h, C.byref(r))
        return {0: None, 2: "rho_end", 3: "max_iter"}.get(r.value, "unknown")

    def state(self) -> dict:
        x = np.zeros(self.n)
        bf, rho, it = C.c_double(), C.c_double(), C.c_int64()
        call("xr_dfo_get", self._h, x.ctypes.data_as(C.c_void_p), C.byref(bf), C.byref(rho), C.byref(it))
        ne = C.c_int64()
        call("xr_dfo_evaluations", self._h, C.byref(ne))
        return {"best_x": x, "best_f": bf.value, "rho": rho.value, "iterations": it.value, "evaluations": ne.value}
