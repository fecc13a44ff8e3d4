"""ctypes binding of oracle/_ref/librefexec.so (test infrastructure only).

One simulation at a time: the reference keeps its state in globals (kernel/Globals.h).
"""
import ctypes as C
import os

import numpy as np

from . import build_refexec

_lib = None


def available():
    return os.path.exists(build_refexec.OUT) or build_refexec.available()


def lib():
    global _lib
    if _lib is None:
        path = build_refexec.build()
        L = C.CDLL(path)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        fp, up = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
        L.refx_create.argtypes = [vp, u32]
        L.refx_create.restype = i32
        L.refx_destroy.argtypes = []
        L.refx_add_particles.argtypes = [u32, fp, fp, fp]
        L.refx_add_particles.restype = i32
        L.refx_step_phase.argtypes = [i32]
        L.refx_step_phase.restype = i32
        L.refx_num_particles.restype = u32
        L.refx_get_state.argtypes = [fp, fp, fp, fp]
        L.refx_get_debug.argtypes = [up, up, up, up, u32, fp, fp, fp]
        L.refx_get_neighbours.argtypes = [u32, up, up, up]
        _lib = L
    return _lib


def _f(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _u(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


class RefExec:
    """The reference step on the CPU.  `width` is the texture width (capacity = width^2)."""

    def __init__(self, params, width):
        self.L = lib()
        self.L.refx_destroy()
        rc = self.L.refx_create(C.byref(params), width)
        if rc:
            raise RuntimeError(f"refx_create rc={rc}")

    def close(self):
        self.L.refx_destroy()

    @property
    def n(self):
        return self.L.refx_num_particles()

    def add_particles(self, pos4, vel4, col4=None):
        pos4 = np.ascontiguousarray(pos4, np.float32)
        vel4 = np.ascontiguousarray(vel4, np.float32)
        col4 = None if col4 is None else np.ascontiguousarray(col4, np.float32)
        rc = self.L.refx_add_particles(len(pos4), _f(pos4), _f(vel4), _f(col4))
        if rc:
            raise RuntimeError(f"refx_add_particles rc={rc}")

    def step_phase(self, phase=0):
        rc = self.L.refx_step_phase(phase)
        if rc:
            raise RuntimeError(f"refx_step_phase rc={rc}")

    def step(self, n=1):
        for _ in range(n):
            self.step_phase(0)

    def state(self):
        n = self.n
        x, v, p, c = (np.zeros((n, 4), np.float32) for _ in range(4))
        self.L.refx_get_state(_f(x), _f(v), _f(p), _f(c))
        return {"x": x, "v": v, "p": p, "col": c}

    def debug(self, ncells=0):
        n = self.n
        keys, perm = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        cs, ce = np.zeros(ncells, np.uint32), np.zeros(ncells, np.uint32)
        lam = np.zeros(n, np.float32)
        fext, om = np.zeros((n, 4), np.float32), np.zeros((n, 4), np.float32)
        self.L.refx_get_debug(_u(keys), _u(perm), _u(cs), _u(ce), ncells, _f(lam), _f(fext), _f(om))
        return {"keys": keys, "perm": perm, "cell_start": cs, "cell_end": ce, "lambda": lam, "fext": fext, "omega": om}

    def neighbours(self, max_entries):
        n = self.n
        lst = np.zeros((n, max_entries), np.uint32)
        cnt, con = np.zeros(n, np.uint32), np.zeros(n, np.uint32)
        self.L.refx_get_neighbours(max_entries, _u(lst), _u(cnt), _u(con))
        return lst, cnt, con
