"""Many independent replicas stepped together (mg_ensemble_*).

`Ensemble(engines)` groups Engines that live on one device; `run(kind,
nstep)` advances every replica by nstep MD (kind 0) or BD (kind 1) steps with
one CUDA graph launch per step.  Each Engine keeps its own state and is read
back as usual (MDRun/BDRun with 0 steps, GetPositions).
"""
import ctypes as C

import numpy as np

from . import abi
from .engine import MolsimError


class Ensemble:
    def __init__(self, engines):
        self.engines = list(engines)
        self.lib = self.engines[0].lib
        arr = (C.c_void_p * len(self.engines))(*[e.h.value for e in self.engines])
        self.h = C.c_void_p()
        st = self.lib.mg_ensemble_create(len(self.engines), arr, C.byref(self.h))
        if st != 0:
            raise MolsimError(st, "ensemble_create")

    def _check(self, st, what):
        if st != 0:
            buf = C.create_string_buffer(512)
            self.lib.mg_ensemble_last_error(self.h, buf, 512)
            raise MolsimError(st, f"{what}: {buf.value.decode(errors='replace')}")

    def run(self, kind, nstep):
        """nstep steps of every replica; returns the device ms of the launches."""
        ms = np.zeros(1)
        self._check(self.lib.mg_ensemble_run(self.h, int(kind), int(nstep), abi.f64(ms)), "ensemble_run")
        return float(ms[0])

    def kernels(self, kind):
        n = np.zeros(1, dtype=np.int32)
        self._check(self.lib.mg_ensemble_kernels(self.h, int(kind), abi.i32(n)), "ensemble_kernels")
        return int(n[0])

    def close(self):
        if self.h:
            self.lib.mg_ensemble_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
