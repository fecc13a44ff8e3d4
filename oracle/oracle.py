"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline / reference arm import
this module; the shipped library never does.  `Oracle(params, capacity, precision)` wraps
one orc_sim of liboracle_f32.so or liboracle_f64.so (see pbd_oracle.c for the semantics).
"""
import ctypes as C
import os

import numpy as np

from . import build_oracle

_LIBS = {}


def _lib(precision):
    if precision not in _LIBS:
        path = build_oracle.targets()[precision]
        if not os.path.exists(path):
            build_oracle.build()
        lib = C.CDLL(path)
        vp, u32, i32, f32p, f64p, u32p = C.c_void_p, C.c_uint32, C.c_int, C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_uint32)
        lib.orc_create.restype = vp
        lib.orc_create.argtypes = [vp, u32]
        lib.orc_destroy.argtypes = [vp]
        lib.orc_set_params.argtypes = [vp, vp]
        lib.orc_add_particles.argtypes = [vp, u32, f32p, f32p, f32p]
        lib.orc_add_particle.argtypes = [vp, f32p, f32p]
        lib.orc_add_particles_mass.argtypes = [vp, u32, f32p, f32p, f32p, f32p]
        lib.orc_clear.argtypes = [vp]
        lib.orc_set_fext.argtypes = [vp, f32p]
        lib.orc_step.argtypes = [vp, i32]
        lib.orc_step_phase.argtypes = [vp, i32]
        lib.orc_num_particles.restype = u32
        lib.orc_num_particles.argtypes = [vp]
        lib.orc_get_state.argtypes = [vp, f64p, f64p, f64p, u32p]
        lib.orc_get_debug.argtypes = [vp, u32p, u32p, u32p, u32p, u32, f64p, f64p, f64p, f64p]
        lib.orc_get_neighbours.argtypes = [vp, u32, u32p, u32p, u32p]
        lib.orc_density_error.argtypes = [vp, f64p]
        lib.orc_expand_bits.restype = u32
        lib.orc_expand_bits.argtypes = [u32]
        lib.orc_morton_f32.restype = u32
        lib.orc_morton_f32.argtypes = [C.c_float, C.c_float, C.c_float]
        lib.orc_set_threads.argtypes = [i32]
        lib.orc_max_threads.restype = i32
        lib.orc_real_size.restype = i32
        lib.orc_render_sprites.argtypes = [f32p, f32p, u32, vp, C.POINTER(C.c_uint8), f32p]
        _LIBS[precision] = lib
    return _LIBS[precision]


def _ptr(a, ctype):
    if a is None:
        return None
    return a.ctypes.data_as(C.POINTER(ctype))


PHASE_ALL, PHASE_FRONT, PHASE_LISTS = 0, 1, 2


class Oracle:
    """One oracle simulation.  `params` is a ctypes pbd_params structure (any object whose
    bytes follow include/pbd.h's layout)."""

    def __init__(self, params, capacity, precision="f64"):
        self.lib = _lib(precision)
        self.precision = precision
        self.params = params
        self.h = self.lib.orc_create(C.byref(params), capacity)
        if not self.h:
            raise MemoryError("orc_create failed")
        self.capacity = capacity

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        rc = self.lib.orc_set_params(self.h, C.byref(params))
        if rc:
            raise RuntimeError(f"orc_set_params rc={rc}")
        self.params = params

    @property
    def n(self):
        return self.lib.orc_num_particles(self.h)

    def add_particles(self, pos4, vel4, col4=None):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        col4 = None if col4 is None else np.ascontiguousarray(col4, dtype=np.float32)
        return self.lib.orc_add_particles(self.h, pos4.shape[0], _ptr(pos4, C.c_float), _ptr(vel4, C.c_float), _ptr(col4, C.c_float))

    def add_particles_mass(self, pos4, vel4, inv_mass, col4=None):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        w = np.ascontiguousarray(inv_mass, dtype=np.float32)
        col4 = None if col4 is None else np.ascontiguousarray(col4, dtype=np.float32)
        return self.lib.orc_add_particles_mass(self.h, pos4.shape[0], _ptr(pos4, C.c_float), _ptr(vel4, C.c_float),
                                               _ptr(col4, C.c_float), _ptr(w, C.c_float))

    def add_particle(self, pos, direction):
        p = np.ascontiguousarray(pos, dtype=np.float32)
        d = np.ascontiguousarray(direction, dtype=np.float32)
        return self.lib.orc_add_particle(self.h, _ptr(p, C.c_float), _ptr(d, C.c_float))

    def clear(self):
        self.lib.orc_clear(self.h)

    def set_fext(self, fext4):
        """f_ext of the current particles in their current order (n, 4)."""
        f = np.ascontiguousarray(fext4, dtype=np.float32)
        assert f.shape == (self.n, 4)
        self.lib.orc_set_fext(self.h, _ptr(f, C.c_float))

    def step(self, nsteps=1):
        rc = self.lib.orc_step(self.h, nsteps)
        if rc:
            raise RuntimeError(f"orc_step rc={rc}")

    def step_phase(self, phase):
        rc = self.lib.orc_step_phase(self.h, phase)
        if rc:
            raise RuntimeError(f"orc_step_phase rc={rc}")

    def state(self):
        n = self.n
        x = np.zeros((n, 4)); v = np.zeros((n, 4)); p = np.zeros((n, 4)); ids = np.zeros(n, np.uint32)
        self.lib.orc_get_state(self.h, _ptr(x, C.c_double), _ptr(v, C.c_double), _ptr(p, C.c_double), _ptr(ids, C.c_uint32))
        return {"x": x, "v": v, "p": p, "ids": ids}

    def debug(self, ncells=0):
        n = self.n
        keys = np.zeros(n, np.uint32); perm = np.zeros(n, np.uint32)
        cs = np.zeros(ncells, np.uint32); ce = np.zeros(ncells, np.uint32)
        lam = np.zeros(n); fext = np.zeros((n, 4)); om = np.zeros((n, 4)); col = np.zeros((n, 4))
        self.lib.orc_get_debug(self.h, _ptr(keys, C.c_uint32), _ptr(perm, C.c_uint32), _ptr(cs, C.c_uint32), _ptr(ce, C.c_uint32),
                               ncells, _ptr(lam, C.c_double), _ptr(fext, C.c_double), _ptr(om, C.c_double), _ptr(col, C.c_double))
        return {"keys": keys, "perm": perm, "cell_start": cs, "cell_end": ce, "lambda": lam, "fext": fext, "omega": om, "col": col}

    def neighbours(self, max_entries):
        n = self.n
        lst = np.zeros((n, max_entries), np.uint32); cnt = np.zeros(n, np.uint32); con = np.zeros(n, np.uint32)
        self.lib.orc_get_neighbours(self.h, max_entries, _ptr(lst, C.c_uint32), _ptr(cnt, C.c_uint32), _ptr(con, C.c_uint32))
        return lst, cnt, con

    def density_error(self):
        out = np.zeros(self.n)
        self.lib.orc_density_error(self.h, _ptr(out, C.c_double))
        return out


def expand_bits(v):
    return _lib("f32").orc_expand_bits(v)


def morton(x, y, z):
    return _lib("f32").orc_morton_f32(x, y, z)


def render_sprites(pos4, col4, cam):
    """The sprite renderer's CPU restatement: (rgba (H, W, 4) uint8 rows top-down, depth (H, W))."""
    pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
    col4 = None if col4 is None else np.ascontiguousarray(col4, dtype=np.float32)
    rgba = np.zeros((cam.height, cam.width, 4), np.uint8)
    depth = np.zeros((cam.height, cam.width), np.float32)
    _lib("f32").orc_render_sprites(_ptr(pos4, C.c_float), _ptr(col4, C.c_float), len(pos4), C.byref(cam),
                                   rgba.ctypes.data_as(C.POINTER(C.c_uint8)), _ptr(depth, C.c_float))
    return rgba, depth


def set_threads(n, precision="f32"):
    _lib(precision).orc_set_threads(n)


def max_threads(precision="f32"):
    return _lib(precision).orc_max_threads()
