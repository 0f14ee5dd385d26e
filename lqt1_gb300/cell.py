"""Host-side mirror of the reference's cell interface for N cells on the GPU.

The reference's boundary is the `Cell` virtual interface implemented by
`TPORd` (SingleCell/Cell.cc:22-42, SingleCell/TPORd.cc:137-376): construct
with a cell type, `setDt`, `setIstim`, `setDVgap_dt`, `update()`, `getV`,
`getDvdt`, `outputAllStates` / `readinAllStates`.  `TPORdCells` offers the same
operations for a whole array of cells at once, through lqt_cells_* of the C ABI.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N

LVEPI, LVENDO, EPI, ENDO, MCELL = N.LVEPI, N.LVENDO, N.EPI, N.ENDO, N.MCELL
STATE_NAMES = ["v", "nai", "nass", "ki", "kss", "cai", "cass", "cansr", "cajsr", "sm", "sh", "sj", "hsp", "jp",
               "mL", "hL", "hLp", "a", "iF", "iS", "ap", "iFp", "iSp", "d", "ff", "fs", "fcaf", "fcas", "jca",
               "nca", "ffp", "fcafp", "xrf", "xrs", "xs1", "xs2", "xk1", "Jrelnp", "Jrelp", "CaMKt"]


def _p(a):
    return None if a is None else a.ctypes.data


class TPORdCells:
    """N TPORd cells (`new TPORd(ct)` for each cell type in `types`)."""

    def __init__(self, types, precision: int = N.MIXED, model: N.Model | str = "default", dt: float = 0.02,
                 stream: int | None = None):
        self.types = np.ascontiguousarray(types, dtype=np.uint8)
        self.n = len(self.types)
        self.precision = precision
        self.model = N.model(model) if isinstance(model, str) else model
        self._dt = dt
        h = C.c_void_p()
        N.check(N.lib().lqt_cells_create(self.n, _p(self.types), precision, C.byref(self.model), dt,
                                         C.c_void_p(stream or 0), C.byref(h)), "lqt_cells_create")
        self._h = h
        self._ist = np.zeros(self.n)
        self._dvgap = np.zeros(self.n)

    def close(self):
        if getattr(self, "_h", None):
            N.lib().lqt_cells_destroy(self._h)
            self._h = None

    __del__ = close

    # TPORd::setDt (TPORd.cc:358) -- fixed at construction here
    @property
    def dt(self):
        return self._dt

    def set_istim(self, ist):
        """setIstim (TPORd.cc:360), per cell or scalar."""
        self._ist = np.ascontiguousarray(np.broadcast_to(np.asarray(ist, np.float64), (self.n,)))
        N.check(N.lib().lqt_cells_set_inputs(self._h, _p(self._ist), _p(self._dvgap)), "lqt_cells_set_inputs")

    def set_dvgap_dt(self, dvgap):
        """setDVgap_dt (TPORd.cc:361), per cell or scalar."""
        self._dvgap = np.ascontiguousarray(np.broadcast_to(np.asarray(dvgap, np.float64), (self.n,)))
        N.check(N.lib().lqt_cells_set_inputs(self._h, _p(self._ist), _p(self._dvgap)), "lqt_cells_set_inputs")

    def update(self, nsteps: int = 1):
        """update() (TPORd.cc:379-1021), nsteps times."""
        N.check(N.lib().lqt_cells_update(self._h, int(nsteps)), "lqt_cells_update")

    def get_v(self):
        out = np.zeros(self.n)
        N.check(N.lib().lqt_cells_get_v(self._h, _p(out)), "lqt_cells_get_v")
        return out

    def get_dvdt(self):
        out = np.zeros(self.n)
        N.check(N.lib().lqt_cells_get_dvdt(self._h, _p(out)), "lqt_cells_get_dvdt")
        return out

    def get_state(self):
        """All states, [n, 40] in outputAllStates order (TPORd.cc:200-252)."""
        out = np.zeros((self.n, N.NSTATE))
        N.check(N.lib().lqt_cells_get_state(self._h, _p(out)), "lqt_cells_get_state")
        return out

    def set_state(self, s):
        s = np.ascontiguousarray(s, dtype=np.float64).reshape(self.n, N.NSTATE)
        N.check(N.lib().lqt_cells_set_state(self._h, _p(s)), "lqt_cells_set_state")

    def get_currents(self):
        """[n, 6] INa, ICaL, IKr, IKs, IK1 (pA/pF) and |dV/dt| (mV/ms) of the
        last update (TPORd getters, SingleCell/TPORd.cc:358-376)."""
        out = np.zeros((self.n, 6))
        N.check(N.lib().lqt_cells_get_currents(self._h, _p(out)), "lqt_cells_get_currents")
        return out

    def output_all_states(self, path: str, i: int = 0, count: int = 1):
        """Text dump of cells [i, i + count) in the reference's format
        (outputAllStates: 40 "%4.10f" lines per cell), through the C ABI."""
        with N.CFile(path, "w") as f:
            N.check(N.lib().lqt_cells_output_states(self._h, i, count, f.ptr), "lqt_cells_output_states")

    def readin_all_states(self, path: str, i: int | None = None, count: int = 1):
        """readinAllStates: 40 values per cell into cells [i, i + count); with
        i = None, one cell's 40 values into every cell."""
        with N.CFile(path, "r") as f:
            if i is not None:
                N.check(N.lib().lqt_cells_readin_states(self._h, i, count, f.ptr), "lqt_cells_readin_states")
                return
            one = np.zeros(N.NSTATE)
            N.check(N.lib().lqt_state_read_text(_p(one), 1, f.ptr), "lqt_state_read_text")
        self.set_state(np.repeat(one[None], self.n, 0))


def initial_state(v0: float = -87.5) -> np.ndarray:
    s = np.zeros(N.NSTATE)
    N.check(N.lib().lqt_initial_state(v0, _p(s)), "lqt_initial_state")
    return s
