"""ctypes binding of libpbd.so (include/pbd.h) for Python callers, tests and bench.py.

The product is the C ABI; this module only marshals arrays.  It fails loudly when the
library is missing: there is no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
# PBD_LIBRARY selects another build of the library (same ABI), e.g. for A/B measurements
LIB_PATH = os.environ.get("PBD_LIBRARY") or os.path.join(HERE, "libpbd.so")

# status codes (include/pbd.h)
OK, ERR_INVALID_ARG, ERR_CAPACITY, ERR_CUDA, ERR_CONFIG, ERR_TIMEOUT, ERR_UNSUPPORTED, ERR_ALLOC, ERR_RANGE = range(9)

ACTIVE = {
    "applyForces": 1 << 0, "findContacts": 1 << 1, "findNeighbours": 1 << 2, "computeLambda": 1 << 3,
    "computeDeltaPositions": 1 << 4, "applyDeltaPositions": 1 << 5, "updatePositions": 1 << 6,
    "computeOmegas": 1 << 7, "computeVorticity": 1 << 8, "computeViscosity": 1 << 9,
}
ACTIVE_ALL = 0x3FF
FLAG_CELL_END_QUIRK, FLAG_TRACK_IDS, FLAG_COLORS, FLAG_FULL_WALK, FLAG_STAGED_PASSES = 1, 2, 4, 8, 32

EXPORTED = [
    "pbd_params_default", "pbd_load_config", "pbd_parse_config", "pbd_write_config", "pbd_validate_params",
    "pbd_create", "pbd_destroy", "pbd_set_params", "pbd_get_params", "pbd_num_particles", "pbd_capacity",
    "pbd_add_particles", "pbd_add_particles_mass", "pbd_add_particles_device", "pbd_add_particle", "pbd_clear", "pbd_step", "pbd_sync",
    "pbd_get_state", "pbd_get_device_state", "pbd_debug_dump", "pbd_debug_neighbours", "pbd_debug_front",
    "pbd_launches_per_step", "pbd_profile_frames", "pbd_sort_keys_noalloc", "pbd_last_error", "pbd_abi_version",
    "pbd_autotune", "pbd_batch_create", "pbd_batch_destroy", "pbd_batch_add_particles", "pbd_batch_step",
    "pbd_batch_sync", "pbd_batch_num_particles", "pbd_batch_get_state", "pbd_batch_autotune",
    "pbd_batch_launches_per_step", "pbd_batch_profile_frames", "pbd_adjoint_forward", "pbd_adjoint_backward", "pbd_render_sprites",
    "pbd_density_error", "pbd_density_error_interior", "pbd_step_readback", "pbd_sort_noalloc_status",
    "pbd_debug_fail_allocations", "pbd_debug_set_wait_limit",
]


class Params(C.Structure):
    """pbd_params (include/pbd.h); mirrors SimulationParameters, kernel/Globals.h:50-75."""
    _fields_ = [
        ("struct_size", C.c_uint32), ("threads_per_block", C.c_uint32), ("particle_radius", C.c_float),
        ("max_neighbours_per_particle", C.c_uint32), ("delta_t", C.c_float), ("gravity", C.c_float),
        ("rest_density", C.c_float), ("kernel_width_spiky", C.c_float), ("k_scorr", C.c_float),
        ("n_scorr", C.c_int32), ("q_scorr", C.c_float), ("c_viscosity", C.c_float),
        ("kernel_width_poly", C.c_float), ("e_vorticity", C.c_float), ("collision_type", C.c_uint32),
        ("kernel_width_neighbours", C.c_uint32), ("max_collision_batches", C.c_uint32), ("stiffness", C.c_float),
        ("enclosure_position_damping", C.c_float), ("enclosure_velocity_damping", C.c_float),
        ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3), ("solver_iterations", C.c_uint32),
        ("stabilization_iterations", C.c_uint32), ("active", C.c_uint32), ("max_grid", C.c_uint32),
        ("lambda_epsilon", C.c_float), ("flags", C.c_uint32),
    ]

    def copy(self):
        p = Params()
        C.memmove(C.byref(p), C.byref(self), C.sizeof(Params))
        return p

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            v = getattr(self, name)
            d[name] = list(v) if not isinstance(v, (int, float)) else v
        return d


class SceneDesc(C.Structure):
    """pbd_scene_desc (include/pbd.h): the per-scene values of a batch."""
    _fields_ = [("capacity", C.c_uint32), ("rest_density", C.c_float), ("gravity", C.c_float),
                ("bounds_min", C.c_float * 3), ("bounds_max", C.c_float * 3)]


class KernelStat(C.Structure):
    _fields_ = [("name", C.c_char * 32), ("launches", C.c_uint32), ("total_ms", C.c_float)]


class Camera(C.Structure):
    """pbd_camera (include/pbd.h): column-major view and projection as glm builds them."""
    _fields_ = [("view", C.c_float * 16), ("projection", C.c_float * 16), ("view_direction", C.c_float * 3),
                ("light_position", C.c_float * 3), ("sphere_radius", C.c_float), ("width", C.c_uint32),
                ("height", C.c_uint32), ("clear_rgba", C.c_float * 4)]


def look_at(eye, center, up):
    """glm::lookAt (right-handed): column-major 4x4 as a (16,) float32 array, and the view direction"""
    eye, center, up = (np.asarray(a, np.float64) for a in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s_ = np.cross(f, up)
    s_ /= np.linalg.norm(s_)
    u = np.cross(s_, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s_, u, -f          # rows of the rotation
    m[0, 3], m[1, 3], m[2, 3] = -s_ @ eye, -u @ eye, f @ eye
    return m.T.astype(np.float32).ravel(), f.astype(np.float32)


def perspective(fovy, aspect, near, far):
    """glm::perspective (radians, right-handed, depth -1..1): column-major (16,) float32"""
    t = np.tan(fovy / 2.0)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = -(far + near) / (far - near)
    m[3, 2] = -1.0
    m[2, 3] = -(2.0 * far * near) / (far - near)
    return m.T.astype(np.float32).ravel()


def camera(eye, center, width, height, fovy=np.pi / 4, near=0.1, far=1000.0, up=(0.0, 1.0, 0.0),
           light=(0.0, 0.0, 10.0), radius=0.5, clear=(0.0, 0.0, 0.0, 1.0)):
    """A pbd_camera looking from `eye` at `center` (the reference's defaults for the rest)."""
    c = Camera()
    v, f = look_at(eye, center, up)
    c.view[:] = v.tolist()
    c.projection[:] = perspective(fovy, width / height, near, far).tolist()
    c.view_direction[:] = f.tolist()
    c.light_position[:] = list(light)
    c.sphere_radius = radius
    c.width, c.height = width, height
    c.clear_rgba[:] = list(clear)
    return c


class PBDError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"pbd error {code}: {msg}")
        self.code = code


_lib = None


def lib():
    """Load libpbd.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise FileNotFoundError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = C.CDLL(LIB_PATH)
        vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int
        fp, u32p = C.POINTER(C.c_float), C.POINTER(C.c_uint32)
        P = C.POINTER(Params)
        sig = {
            "pbd_params_default": [P], "pbd_load_config": [P, C.c_char_p], "pbd_parse_config": [P, C.c_char_p, C.c_char_p],
            "pbd_write_config": [P, C.c_char_p], "pbd_validate_params": [P],
            "pbd_create": [P, u32, C.POINTER(vp)], "pbd_destroy": [vp], "pbd_set_params": [vp, P],
            "pbd_get_params": [vp, P], "pbd_num_particles": [vp, u32p], "pbd_capacity": [vp, u32p],
            "pbd_add_particles": [vp, u32, fp, fp, fp], "pbd_add_particles_device": [vp, u32, vp, vp, vp, vp],
            "pbd_add_particles_mass": [vp, u32, fp, fp, fp, fp],
            "pbd_add_particle": [vp, fp, fp], "pbd_clear": [vp], "pbd_step": [vp, i32, vp], "pbd_sync": [vp],
            "pbd_get_state": [vp, fp, fp, fp, u32p],
            "pbd_step_readback": [vp, C.c_int, vp, C.POINTER(fp), C.POINTER(fp)], "pbd_get_device_state": [vp, C.POINTER(vp), C.POINTER(vp), C.POINTER(vp)],
            "pbd_debug_dump": [vp, u32p, u32p, u32p, u32p, u32, fp, fp, fp],
            "pbd_debug_neighbours": [vp, u32, u32p, u32p, u32p, i32], "pbd_debug_front": [vp, vp],
            "pbd_launches_per_step": [vp, u32p],
            "pbd_profile_frames": [vp, i32, vp, C.POINTER(KernelStat), u32, u32p],
            "pbd_sort_keys_noalloc": [vp, vp, vp, u32, u32, vp], "pbd_sort_noalloc_status": [vp],
            "pbd_debug_fail_allocations": [u32, u32], "pbd_debug_set_wait_limit": [vp, u32, i32],
            "pbd_autotune": [vp, C.c_char_p, vp, u32p],
            "pbd_batch_create": [P, u32, C.POINTER(SceneDesc), C.POINTER(vp)], "pbd_batch_destroy": [vp],
            "pbd_batch_add_particles": [vp, u32, u32, fp, fp], "pbd_batch_step": [vp, i32, vp],
            "pbd_batch_sync": [vp], "pbd_batch_num_particles": [vp, u32, u32p],
            "pbd_batch_get_state": [vp, u32, fp, fp], "pbd_batch_autotune": [vp, C.c_char_p, vp, u32p],
            "pbd_batch_launches_per_step": [vp, u32p],
            "pbd_batch_profile_frames": [vp, i32, vp, C.POINTER(KernelStat), u32, u32p],
            "pbd_adjoint_forward": [vp, i32, i32, vp],
            "pbd_render_sprites": [vp, C.POINTER(Camera), C.POINTER(C.c_uint8), fp, vp],
            "pbd_density_error": [vp, fp, C.POINTER(C.c_double), C.POINTER(C.c_double), vp],
            "pbd_density_error_interior": [vp, u32, C.c_float, C.POINTER(C.c_double), C.POINTER(C.c_double), u32p, vp],
            "pbd_adjoint_backward": [vp, fp, fp, fp, C.POINTER(C.c_double), C.POINTER(C.c_double), vp],
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.argtypes = args
            f.restype = i32
        L.pbd_last_error.restype = C.c_char_p
        L.pbd_last_error.argtypes = []
        L.pbd_abi_version.restype = u32
        L.pbd_abi_version.argtypes = []
        _lib = L
    return _lib


def check(rc):
    if rc != OK:
        raise PBDError(rc, lib().pbd_last_error().decode(errors="replace"))
    return rc


def default_params():
    p = Params()
    check(lib().pbd_params_default(C.byref(p)))
    return p


def load_config(path, params=None):
    p = default_params() if params is None else params.copy()
    check(lib().pbd_load_config(C.byref(p), os.fsencode(path)))
    return p


def parse_config(text, params=None, base_dir=None):
    p = default_params() if params is None else params.copy()
    check(lib().pbd_parse_config(C.byref(p), text.encode(), None if base_dir is None else os.fsencode(base_dir)))
    return p


def _fp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_float))


def _up(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_uint32))


class Sim:
    """One pbd_sim handle (the reference's Fluid object plus its injection callbacks)."""

    def __init__(self, params, capacity):
        self.L = lib()
        self.h = C.c_void_p()
        check(self.L.pbd_create(C.byref(params), capacity, C.byref(self.h)))
        self.capacity = capacity

    def close(self):
        if self.h:
            self.L.pbd_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n(self):
        v = C.c_uint32()
        check(self.L.pbd_num_particles(self.h, C.byref(v)))
        return v.value

    def params(self):
        p = Params()
        check(self.L.pbd_get_params(self.h, C.byref(p)))
        return p

    def set_params(self, p):
        check(self.L.pbd_set_params(self.h, C.byref(p)))

    def add_particles(self, pos4, vel4, col4=None):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        col4 = None if col4 is None else np.ascontiguousarray(col4, dtype=np.float32)
        check(self.L.pbd_add_particles(self.h, pos4.shape[0], _fp(pos4), _fp(vel4), _fp(col4)))

    def add_particles_mass(self, pos4, vel4, inv_mass, col4=None):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        w = np.ascontiguousarray(inv_mass, dtype=np.float32)
        col4 = None if col4 is None else np.ascontiguousarray(col4, dtype=np.float32)
        check(self.L.pbd_add_particles_mass(self.h, pos4.shape[0], _fp(pos4), _fp(vel4), _fp(col4), _fp(w)))

    def add_particle(self, pos, direction):
        p = np.ascontiguousarray(pos, dtype=np.float32)
        d = np.ascontiguousarray(direction, dtype=np.float32)
        check(self.L.pbd_add_particle(self.h, _fp(p), _fp(d)))

    def clear(self):
        check(self.L.pbd_clear(self.h))

    def step(self, nsteps=1, stream=0):
        check(self.L.pbd_step(self.h, nsteps, C.c_void_p(stream)))

    def sync(self):
        check(self.L.pbd_sync(self.h))

    def step_readback(self, nsteps=1, stream=0, copy=True):
        """pbd_step, then the final x and v ((n, 4) float32 each) from the library's pinned host
        arrays (views valid until the next call unless `copy`)."""
        px, pv = C.POINTER(C.c_float)(), C.POINTER(C.c_float)()
        check(self.L.pbd_step_readback(self.h, nsteps, C.c_void_p(stream), C.byref(px), C.byref(pv)))
        n = self.n
        x = np.ctypeslib.as_array(px, shape=(n, 4))
        v = np.ctypeslib.as_array(pv, shape=(n, 4))
        return (x.copy(), v.copy()) if copy else (x, v)

    def state(self):
        n = self.n
        x = np.zeros((n, 4), np.float32); v = np.zeros((n, 4), np.float32)
        p = np.zeros((n, 4), np.float32); ids = np.zeros(n, np.uint32)
        check(self.L.pbd_get_state(self.h, _fp(x), _fp(v), _fp(p), _up(ids)))
        return {"x": x, "v": v, "p": p, "ids": ids}

    def debug(self, ncells=0):
        n = self.n
        keys = np.zeros(n, np.uint32); perm = np.zeros(n, np.uint32)
        cs = np.zeros(ncells, np.uint32); ce = np.zeros(ncells, np.uint32)
        lam = np.zeros(n, np.float32); fext = np.zeros((n, 4), np.float32); om = np.zeros((n, 4), np.float32)
        check(self.L.pbd_debug_dump(self.h, _up(keys), _up(perm), _up(cs), _up(ce), ncells, _fp(lam), _fp(fext), _fp(om)))
        return {"keys": keys, "perm": perm, "cell_start": cs, "cell_end": ce, "lambda": lam, "fext": fext, "omega": om}

    def neighbours(self, max_entries, walker=0):
        n = self.n
        lst = np.zeros((n, max_entries), np.uint32); cnt = np.zeros(n, np.uint32); con = np.zeros(n, np.uint32)
        check(self.L.pbd_debug_neighbours(self.h, max_entries, _up(lst), _up(cnt), _up(con), walker))
        return lst, cnt, con

    def front(self, stream=0):
        check(self.L.pbd_debug_front(self.h, C.c_void_p(stream)))

    def autotune(self, cache_path=None, stream=0):
        """Threads per block of the neighbour passes (64, 128 or 256), timed on this simulation
        (which advances frames) unless `cache_path` already holds this workload."""
        b = C.c_uint32()
        check(self.L.pbd_autotune(self.h, None if cache_path is None else os.fsencode(cache_path),
                                  C.c_void_p(stream), C.byref(b)))
        return b.value

    def profile(self, nsteps, stream=0):
        """{kernel name: (launches, total device ms)} over `nsteps` directly launched frames."""
        stats = (KernelStat * 32)()
        n = C.c_uint32()
        check(self.L.pbd_profile_frames(self.h, nsteps, C.c_void_p(stream), stats, 32, C.byref(n)))
        return {stats[k].name.decode(): (stats[k].launches, stats[k].total_ms) for k in range(n.value)}

    def device_state(self):
        x, v, p = C.c_void_p(), C.c_void_p(), C.c_void_p()
        check(self.L.pbd_get_device_state(self.h, C.byref(x), C.byref(v), C.byref(p)))
        return x.value, v.value, p.value

    def launches_per_step(self):
        v = C.c_uint32()
        check(self.L.pbd_launches_per_step(self.h, C.byref(v)))
        return v.value

    def render(self, cam, stream=0):
        """(rgba (H, W, 4) uint8 rows top-down, depth (H, W) float32) of the particle sprites"""
        rgba = np.zeros((cam.height, cam.width, 4), np.uint8)
        depth = np.zeros((cam.height, cam.width), np.float32)
        check(self.L.pbd_render_sprites(self.h, C.byref(cam), rgba.ctypes.data_as(C.POINTER(C.c_uint8)), _fp(depth),
                                        C.c_void_p(stream)))
        return rgba, depth

    def density_error(self, stream=0):
        """(C_i per particle in the current order, mean |C|, max |C|) after the last frame"""
        err = np.zeros(self.n, np.float32)
        mean, mx = C.c_double(), C.c_double()
        check(self.L.pbd_density_error(self.h, _fp(err), C.byref(mean), C.byref(mx), C.c_void_p(stream)))
        return err, mean.value, mx.value

    def density_error_interior(self, min_neighbours, margin, stream=0):
        """(mean |C|, max |C|, particles counted) over the interior particles: list length >=
        min_neighbours and more than `margin` inside the enclosure on every axis"""
        mean, mx, n = C.c_double(), C.c_double(), C.c_uint32()
        check(self.L.pbd_density_error_interior(self.h, min_neighbours, margin, C.byref(mean), C.byref(mx), C.byref(n),
                                                C.c_void_p(stream)))
        return mean.value, mx.value, n.value

    def adjoint_forward(self, nsteps, ckpt_every, stream=0):
        check(self.L.pbd_adjoint_forward(self.h, nsteps, ckpt_every, C.c_void_p(stream)))

    def adjoint_backward(self, dl_dx_final, stream=0):
        """Returns (dL/dv0, dL/dx0, dL/drest_density, dL/deps); arrays in the pre-forward order."""
        g = np.ascontiguousarray(dl_dx_final, dtype=np.float32)
        n = self.n
        dv = np.zeros((n, 4), np.float32)
        dx = np.zeros((n, 4), np.float32)
        dr, de = C.c_double(), C.c_double()
        check(self.L.pbd_adjoint_backward(self.h, _fp(g), _fp(dv), _fp(dx), C.byref(dr), C.byref(de), C.c_void_p(stream)))
        return dv, dx, dr.value, de.value


class Batch:
    """A pbd_batch: many independent scenes stepped together."""

    def __init__(self, shared_params, scene_descs):
        self.L = lib()
        self.h = C.c_void_p()
        arr = (SceneDesc * len(scene_descs))(*scene_descs)
        check(self.L.pbd_batch_create(C.byref(shared_params), len(scene_descs), arr, C.byref(self.h)))
        self.nscenes = len(scene_descs)

    def close(self):
        if self.h:
            self.L.pbd_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_particles(self, scene, pos4, vel4):
        pos4 = np.ascontiguousarray(pos4, dtype=np.float32)
        vel4 = np.ascontiguousarray(vel4, dtype=np.float32)
        check(self.L.pbd_batch_add_particles(self.h, scene, pos4.shape[0], _fp(pos4), _fp(vel4)))

    def step(self, nsteps=1, stream=0):
        check(self.L.pbd_batch_step(self.h, nsteps, C.c_void_p(stream)))

    def sync(self):
        check(self.L.pbd_batch_sync(self.h))

    def count(self, scene):
        v = C.c_uint32()
        check(self.L.pbd_batch_num_particles(self.h, scene, C.byref(v)))
        return v.value

    def state(self, scene):
        n = self.count(scene)
        x = np.zeros((n, 4), np.float32)
        v = np.zeros((n, 4), np.float32)
        check(self.L.pbd_batch_get_state(self.h, scene, _fp(x), _fp(v)))
        return {"x": x, "v": v}

    def autotune(self, cache_path=None, stream=0):
        b = C.c_uint32()
        check(self.L.pbd_batch_autotune(self.h, None if cache_path is None else os.fsencode(cache_path),
                                        C.c_void_p(stream), C.byref(b)))
        return b.value

    def launches_per_step(self):
        v = C.c_uint32()
        check(self.L.pbd_batch_launches_per_step(self.h, C.byref(v)))
        return v.value

    def profile(self, nsteps, stream=0):
        stats = (KernelStat * 32)()
        n = C.c_uint32()
        check(self.L.pbd_batch_profile_frames(self.h, nsteps, C.c_void_p(stream), stats, 32, C.byref(n)))
        return {stats[k].name.decode(): (stats[k].launches, stats[k].total_ms) for k in range(n.value)}


def scene_desc(capacity, rest_density, gravity, box):
    d = SceneDesc()
    d.capacity = capacity
    d.rest_density = rest_density
    d.gravity = gravity
    for a in range(3):
        d.bounds_min[a] = 1.5
        d.bounds_max[a] = float(box) - 1.5
    return d
