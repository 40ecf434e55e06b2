"""vkxpbd — GB300 (sm_103a) drop-in for the reference's `vkxpbd` pybind11 module.

Same names, argument meanings, defaults and error messages as the reference's
bindings (src/bindings.cpp:8-300): `SolverConfig`, `XpbdSolver`,
`enumerate_devices`. The work is done by libxpbd_gb300.so (CUDA kernels for
sm_103a behind the C ABI declared in include/xpbd.h); this module only
converts numpy arrays and forwards calls. There is no CPU fallback: importing
the module fails if the library cannot be loaded or built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _abi

__all__ = ["SolverConfig", "XpbdSolver", "enumerate_devices", "lib_path", "NUM_CELLS"]
__version__ = "0.1.0"

NUM_CELLS = 128 ** 3
_lib = _abi.load()


def lib_path() -> str:
    return _abi.LIB_PATH


def _check(rc: int) -> None:
    if rc != 0:
        raise RuntimeError(_lib.xpbd_last_error().decode("utf-8", "replace"))


def _f32(a) -> np.ndarray:  # py::array_t<float, c_style | forcecast>
    return np.ascontiguousarray(a, dtype=np.float32)


def _u32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.uint32)


def _i32(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.int32)


def _ptr(a, t):
    return None if a is None else a.ctypes.data_as(t)


_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)
_UP = C.POINTER(C.c_uint32)

_FIELDS = [  # (name, ctype kind) of vkx::SolverConfig, src/scene.h:15-40
    ("dt", float), ("substeps", int), ("iterations", int), ("particle_v_max", float),
    ("soft_contact_mu", float), ("shape_material_mu", float), ("soft_contact_relaxation", float),
    ("particle_adhesion", float), ("particle_mu", float), ("particle_cohesion", float),
    ("particle_max_radius", float), ("search_radius", float), ("soft_contact_margin", float),
    ("enable_restitution", bool), ("soft_contact_restitution", float), ("has_ground_plane", bool),
    ("ground_plane_altitude", float), ("shader_dir", str), ("device_index", int), ("compat_mode", bool),
    ("enable_validation", bool), ("enable_diagnostics", bool), ("enable_profile", bool),
    ("max_diag_pairs", int), ("substep_batch_size", int),
]


class SolverConfig:
    """vkx::SolverConfig with the reference's defaults (src/scene.h:14-41).
    `shader_dir`, `compat_mode` and `enable_validation` are accepted and ignored."""

    __slots__ = ("_c",)

    def __init__(self):
        object.__setattr__(self, "_c", _abi.Config())
        _lib.xpbd_config_default(C.byref(self._c))

    def __getattr__(self, name):
        kinds = dict(_FIELDS)
        if name not in kinds:
            raise AttributeError(name)
        v = getattr(self._c, name)
        if kinds[name] is bool:
            return bool(v)
        if kinds[name] is str:
            return v.decode("utf-8")
        return v

    def __setattr__(self, name, value):
        if name == "gravity":
            type(self).gravity.fset(self, value)
            return
        kinds = dict(_FIELDS)
        if name not in kinds:
            raise AttributeError(f"'SolverConfig' object has no attribute '{name}'")
        k = kinds[name]
        if k is str:
            b = str(value).encode("utf-8")[:255]
            setattr(self._c, name, b)
        elif k is bool:
            setattr(self._c, name, 1 if bool(value) else 0)
        elif k is int:
            setattr(self._c, name, int(value))
        else:
            setattr(self._c, name, float(value))

    @property
    def gravity(self):  # bindings.cpp:38-46
        return [float(self._c.gravity[0]), float(self._c.gravity[1]), float(self._c.gravity[2])]

    @gravity.setter
    def gravity(self, g):
        g = list(g)
        if len(g) >= 3:
            self._c.gravity[0], self._c.gravity[1], self._c.gravity[2] = float(g[0]), float(g[1]), float(g[2])

    def __repr__(self):
        items = ", ".join(f"{n}={getattr(self, n)!r}" for n, _ in _FIELDS)
        return f"SolverConfig({items}, gravity={self.gravity!r})"


def enumerate_devices():
    """Names of the visible CUDA devices (the reference lists Vulkan devices)."""
    n = C.c_int(0)
    _check(_lib.xpbd_device_count(C.byref(n)))
    out = []
    buf = C.create_string_buffer(256)
    for i in range(n.value):
        _check(_lib.xpbd_device_name(i, buf, 256))
        out.append(buf.value.decode("utf-8", "replace"))
    return out


def debug_lookback_hold(hold_tile: int, wait_ns: int = 1_000_000) -> None:
    """Test hook of the sort's bounded look-back wait (xpbd_debug_lookback_hold): tile
    `hold_tile` of the first radix pass of every later particle sort never publishes, so
    the next step fails with "device wait timed out" after wait_ns. hold_tile < 0 restores
    normal operation."""
    _check(_lib.xpbd_debug_lookback_hold(int(hold_tile), int(wait_ns)))


class XpbdSolver:
    """vkx::XpbdSolver (src/scene.h:74-135) on the GPU."""

    def __init__(self):
        h = C.c_void_p()
        _check(_lib.xpbd_create(C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            _lib.xpbd_destroy(h)
            self._h = None

    # ---- scene build --------------------------------------------------------
    def init(self, config, num_particles, max_contacts=0):
        _check(_lib.xpbd_init(self._h, C.byref(config._c), int(num_particles), int(max_contacts)))

    # ---- rigid bodies (extension; one body per mesh) ------------------------------
    def set_bodies(self, q=None, qd=None, com=None, inertia=None, inv_inertia=None, inv_mass=None, flags=None):
        """Body table, one row per mesh (xpbd_set_bodies): q (nb, 7) position + quaternion xyzw,
        qd (nb, 6) linear + angular velocity, com (nb, 3), inertia / inv_inertia (nb, 3, 3),
        inv_mass (nb,), flags (nb,). None keeps the current values. Bodies with inv_mass > 0
        are dynamic and their meshes are in the body frame."""
        nb = self.mesh_count
        arrs = [None if a is None else _f32(a).reshape(-1) for a in (q, qd, com, inertia, inv_inertia, inv_mass)]
        fl = None if flags is None else _i32(flags).reshape(-1)
        _check(_lib.xpbd_set_bodies(self._h, *[_ptr(a, _FP) for a in arrs], _ptr(fl, _IP), nb))

    def set_body_scenes(self, scenes):
        """Batched solvers: the scene of each body (one per mesh), -1 for static bodies
        shared by every scene (xpbd_set_body_scenes)."""
        sc = _i32(scenes).reshape(-1)
        _check(_lib.xpbd_set_body_scenes(self._h, _ptr(sc, _IP), sc.size))

    def get_body_q(self):
        nb = self.mesh_count
        q = np.zeros((nb, 7), np.float32)
        _check(_lib.xpbd_get_bodies(self._h, _ptr(q, _FP), None, nb))
        return q

    def get_body_qd(self):
        nb = self.mesh_count
        qd = np.zeros((nb, 6), np.float32)
        _check(_lib.xpbd_get_bodies(self._h, None, _ptr(qd, _FP), nb))
        return qd

    def set_body_params(self, **kw):
        """angular_damping, rigid_contact_margin, rigid_contact_relaxation,
        rigid_contact_con_weighting, rigid_mu_torsional, rigid_mu_rolling,
        particle_contact_con_weighting."""
        bp = _abi.BodyParams()
        _lib.xpbd_body_params_default(C.byref(bp))
        for k, v in kw.items():
            if not hasattr(bp, k):
                raise AttributeError(k)
            setattr(bp, k, v)
        _check(_lib.xpbd_set_body_params(self._h, C.byref(bp)))

    def record_start(self, directory, first_frame=1):
        """Write the positions after every later step to directory/frame_%04d.npy from a
        writer thread (the add-on's cache, overlapped with the next frame)."""
        _check(_lib.xpbd_record_start(self._h, os.fsencode(directory), int(first_frame)))

    def record_stop(self):
        """Wait for pending files; returns how many were written."""
        k = C.c_int(0)
        _check(_lib.xpbd_record_stop(self._h, C.byref(k)))
        return int(k.value)

    def autotune(self):
        """Pick the fastest sort variant on the current keys (xpbd_autotune)."""
        best = (C.c_int * 2)()
        names = ["8b x2", "8b x4", "8b x8", "8b x16", "7b x4", "7b x8", "7b x16", "7b x32"]
        t = (C.c_double * len(names))()
        _check(_lib.xpbd_autotune(self._h, best, t))
        return {"bits": int(best[0]), "keys_per_thread": int(best[1]),
                "sort_us": {names[k]: float(t[k]) for k in range(len(names))}}

    def set_sort_variant(self, bits, keys_per_thread):
        _check(_lib.xpbd_set_sort_variant(self._h, int(bits), int(keys_per_thread)))

    def set_solve_split(self, mode):
        """First iteration against contact generation: 0 fused after it, 1 particle-particle
        part beside it, -1 (default) timed on the first frames (xpbd_set_solve_split)."""
        _check(_lib.xpbd_set_solve_split(self._h, int(mode)))

    @property
    def solve_split(self):
        """The form in use: 0 fused, 1 split, -1 not decided yet."""
        v = C.c_int(0)
        _check(_lib.xpbd_get_solve_split(self._h, C.byref(v)))
        return int(v.value)

    def set_solve_form(self, form):
        """Solve-kernel form: 0 per-thread pair terms, 1 warp pair pass, 2 per-thread from a
        block's neighbourhood staged in shared memory, 3 one warp per particle, -1 (default)
        3 for small scenes, else 0 or 1 timed on the scene's own substeps
        (xpbd_set_solve_form). Results are identical."""
        _check(_lib.xpbd_set_solve_form(self._h, int(form)))

    @property
    def solve_form(self):
        """The solve-kernel form in use (0-3; see set_solve_form)."""
        v = C.c_int(0)
        _check(_lib.xpbd_get_solve_form(self._h, C.byref(v)))
        return int(v.value)

    def update_config(self, config):
        """New contact / material parameters after init (xpbd_update_config)."""
        _check(_lib.xpbd_update_config(self._h, C.byref(config._c)))

    # ---- differentiable rollout (extension) -----------------------------------------
    def rollout(self, dt, substeps, frames, iterations=1, checkpoint_frames=2):
        """Step `frames` frames (like step) keeping checkpoints for rollout_backward."""
        _check(_lib.xpbd_rollout(self._h, float(dt), int(substeps), int(iterations), int(frames),
                                 int(checkpoint_frames)))

    def rollout_backward(self, grad_x_final, grad_v_final=None):
        """Adjoint of the last rollout: dict of float32 gradients w.r.t. the initial
        positions 'x0' (n, 3), velocities 'v0' (n, 3), inverse masses 'inv_mass' (n,) and the
        float64 scalars 'soft_contact_mu', 'shape_material_mu', 'particle_mu',
        'soft_contact_restitution'."""
        n = self.particle_count
        gx = _f32(grad_x_final).reshape(-1)
        gv = None if grad_v_final is None else _f32(grad_v_final).reshape(-1)
        out_x = np.zeros((n, 3), np.float32)
        out_v = np.zeros((n, 3), np.float32)
        out_w = np.zeros(n, np.float32)
        params = (C.c_double * 4)()
        _check(_lib.xpbd_rollout_backward(self._h, _ptr(gx, _FP), _ptr(gv, _FP), _ptr(out_x, _FP),
                                          _ptr(out_v, _FP), _ptr(out_w, _FP), params))
        return {"x0": out_x, "v0": out_v, "inv_mass": out_w, "soft_contact_mu": params[0],
                "shape_material_mu": params[1], "particle_mu": params[2], "soft_contact_restitution": params[3]}

    def init_batched(self, config, scene_counts, max_contacts=0):
        """Independent scenes stepped together (xpbd_batch_init). Particle arrays passed to
        set_particles and returned by the getters are the scenes' particles concatenated in
        scene order; scene_offsets() gives where each scene starts."""
        counts = [int(c) for c in scene_counts]
        arr = (C.c_size_t * max(len(counts), 1))(*counts)
        _check(_lib.xpbd_batch_init(self._h, C.byref(config._c), arr, len(counts), int(max_contacts)))

    def scene_count(self):
        return int(_lib.xpbd_batch_scene_count(self._h))

    def scene_offsets(self):
        k = self.scene_count()
        out = (C.c_size_t * (k + 1))()
        _check(_lib.xpbd_batch_scene_offsets(self._h, out, k + 1))
        return np.array(out[:], dtype=np.int64)

    def add_mesh(self, vertices, indices, shape_margin=0.0, shape_rot=None, is_watertight=None):
        v = _f32(vertices).reshape(-1)
        t = _u32(indices).reshape(-1)
        rot = None if shape_rot is None else _f32(shape_rot).reshape(-1)
        wt = -1 if is_watertight is None else (1 if bool(is_watertight) else 0)
        _check(_lib.xpbd_add_mesh(self._h, _ptr(v, _FP), v.size // 3, _ptr(t, _UP), t.size // 3,
                                  float(shape_margin), _ptr(rot, _FP), wt))

    def finalize_meshes(self):
        _check(_lib.xpbd_finalize_meshes(self._h))

    def set_particles(self, q, qd=None, inv_mass=None, radii=None, flags=None):
        q = _f32(q).reshape(-1)
        n = q.size // 3
        qd = None if qd is None else _f32(qd).reshape(-1)
        w = None if inv_mass is None else _f32(inv_mass).reshape(-1)
        r = None if radii is None else _f32(radii).reshape(-1)
        fl = None if flags is None else _i32(flags).reshape(-1)
        for a in (qd,):
            if a is not None and a.size < n * 3:
                raise RuntimeError("set_particles: qd is shorter than q")
        for a in (w, r, fl):
            if a is not None and a.size < n:
                raise RuntimeError("set_particles: per-particle array is shorter than the particle count")
        _check(_lib.xpbd_set_particles(self._h, _ptr(q, _FP), _ptr(qd, _FP), _ptr(w, _FP), _ptr(r, _FP),
                                       _ptr(fl, _IP), n))

    def update_mesh(self, mesh_index, verts, velocities=None):
        v = _f32(verts).reshape(-1)
        nv = v.size // 3
        vel = None
        if velocities is not None:
            vel = _f32(velocities).reshape(-1)
            if vel.size == 0:
                vel = None
            elif vel.size // 3 != nv:
                raise RuntimeError("update_mesh: velocities size mismatch with vertices")
        _check(_lib.xpbd_update_mesh(self._h, int(mesh_index), _ptr(v, _FP), nv, _ptr(vel, _FP)))

    # ---- stepping -------------------------------------------------------------
    def step(self, dt=1.0 / 60.0, substeps=1, iterations=2):
        _check(_lib.xpbd_step(self._h, float(dt), int(substeps), int(iterations)))

    def collide_only(self):
        _check(_lib.xpbd_collide_only(self._h))

    def step_solve_only(self, dt, substeps, iterations):
        _check(_lib.xpbd_step_solve_only(self._h, float(dt), int(substeps), int(iterations)))

    # ---- state ------------------------------------------------------------------
    def get_positions(self):
        n = self.particle_count
        out = np.empty((n, 3), np.float32)
        _check(_lib.xpbd_get_positions(self._h, _ptr(out, _FP), n))
        return out

    def get_velocities(self):
        n = self.particle_count
        out = np.empty((n, 3), np.float32)
        _check(_lib.xpbd_get_velocities(self._h, _ptr(out, _FP), n))
        return out

    @property
    def particle_count(self):
        return int(_lib.xpbd_particle_count(self._h))

    @property
    def mesh_count(self):
        return int(_lib.xpbd_mesh_count(self._h))

    @property
    def last_contact_count(self):
        return int(_lib.xpbd_last_contact_count(self._h))

    # ---- contacts ---------------------------------------------------------------
    def _contacts(self, which):
        m = max(self.last_contact_count, 0)
        vec = which in ("normals", "body_positions", "body_velocities")
        out = np.empty((m, 3) if vec else m, np.float32 if vec else np.int32)
        if m == 0:
            return out
        args = {k: None for k in ("particles", "shapes", "normals", "body_positions", "body_velocities")}
        args[which] = out
        _check(_lib.xpbd_get_contacts(self._h, _ptr(args["particles"], _IP), _ptr(args["shapes"], _IP),
                                      _ptr(args["normals"], _FP), _ptr(args["body_positions"], _FP),
                                      _ptr(args["body_velocities"], _FP)))
        return out

    def get_contact_particles(self):
        return self._contacts("particles")

    def get_contact_shapes(self):
        return self._contacts("shapes")

    def get_contact_normals(self):
        return self._contacts("normals")

    def get_contact_body_positions(self):
        return self._contacts("body_positions")

    def get_contact_body_velocities(self):
        return self._contacts("body_velocities")

    def set_contact_data(self, particles, shapes, body_positions, normals, contact_count):
        c = int(contact_count)
        p = _i32(particles).reshape(-1)
        s = _i32(shapes).reshape(-1)
        bp = _f32(body_positions).reshape(-1)
        nn = _f32(normals).reshape(-1)
        if c > 0 and (p.size < c or s.size < c or bp.size < 3 * c or nn.size < 3 * c):
            raise RuntimeError("set_contact_data: arrays shorter than contact_count")
        _check(_lib.xpbd_set_contact_data(self._h, _ptr(p, _IP), _ptr(s, _IP), _ptr(bp, _FP), _ptr(nn, _FP), c))

    # ---- hash grid / solver debug getters ----------------------------------------
    def get_sorted_cells(self):
        n = self.particle_count
        out = np.empty(n, np.uint32)
        if n:
            _check(_lib.xpbd_get_sorted_cells(self._h, _ptr(out, _UP), n))
        return out

    def get_sorted_point_ids(self):
        n = self.particle_count
        out = np.empty(n, np.uint32)
        if n:
            _check(_lib.xpbd_get_sorted_point_ids(self._h, _ptr(out, _UP), n))
        return out

    def get_cell_starts(self):
        out = np.empty(NUM_CELLS, np.int32)
        _check(_lib.xpbd_get_cell_starts(self._h, _ptr(out, _IP), NUM_CELLS))
        return out

    def get_cell_ends(self):
        out = np.empty(NUM_CELLS, np.int32)
        _check(_lib.xpbd_get_cell_ends(self._h, _ptr(out, _IP), NUM_CELLS))
        return out

    def get_deltas(self):
        n = self.particle_count
        out = np.empty((n, 3), np.float32)
        if n:
            _check(_lib.xpbd_get_deltas(self._h, _ptr(out, _FP), n))
        return out

    # ---- diagnostics ----------------------------------------------------------
    def get_diag_pair_count(self):
        v = C.c_uint32(0)
        _check(_lib.xpbd_get_diag_pair_count(self._h, C.byref(v)))
        return int(v.value)

    def get_diag_overflow_count(self):
        v = C.c_uint32(0)
        _check(_lib.xpbd_get_diag_overflow_count(self._h, C.byref(v)))
        return int(v.value)

    def reset_diag_buffers(self):
        _check(_lib.xpbd_reset_diag_buffers(self._h))

    def get_diag_pairs(self):
        cnt = C.c_size_t(0)
        _check(_lib.xpbd_get_diag_pairs(self._h, None, 0, C.byref(cnt)))
        k = cnt.value
        if k == 0:
            return []
        buf = (_abi.PairRecord * k)()
        _check(_lib.xpbd_get_diag_pairs(self._h, buf, k, C.byref(cnt)))
        out = []
        for r in buf:  # bindings.cpp:242-263
            out.append({
                "i": int(r.i), "j": int(r.j), "dist": float(r.dist), "err": float(r.err),
                "normal": tuple(float(x) for x in r.normal), "vrel": tuple(float(x) for x in r.vrel),
                "vn": float(r.vn), "vt_len": float(r.vt_len), "denom": float(r.denom),
                "lambda_n": float(r.lambda_n), "lambda_f": float(r.lambda_f),
                "delta_i": tuple(float(x) for x in r.delta_i), "iter_index": int(r.iter_index),
            })
        return out

    def _aux(self, which, dtype):
        cnt = C.c_size_t(0)
        _check(_lib.xpbd_get_aux_diag(self._h, which, None, 0, C.byref(cnt)))
        out = np.zeros(cnt.value, dtype)
        if cnt.value:
            _check(_lib.xpbd_get_aux_diag(self._h, which, out.ctypes.data_as(C.c_void_p), cnt.value, C.byref(cnt)))
        return out

    def get_p11_diag(self):
        return self._aux(0, np.uint32)

    def get_p11_apply_diag(self):
        return self._aux(1, np.uint32)

    def get_shape_contact_diag(self):
        return self._aux(2, np.float32)

    def get_mesh_candidate_diag(self):
        return self._aux(3, np.uint32)

    def _bvh(self, mesh_index, lower):
        k = C.c_size_t(0)
        _check(_lib.xpbd_get_mesh_bvh(self._h, int(mesh_index), None, None, 0, C.byref(k)))
        lo = np.zeros((k.value, 4), np.float32)
        hi = np.zeros((k.value, 4), np.float32)
        if k.value:
            _check(_lib.xpbd_get_mesh_bvh(self._h, int(mesh_index), _ptr(lo, _FP), _ptr(hi, _FP), k.value,
                                          C.byref(k)))
        return lo if lower else hi

    def get_mesh_bvh_lowers(self, mesh_index):
        return self._bvh(mesh_index, True)

    def get_mesh_bvh_uppers(self, mesh_index):
        return self._bvh(mesh_index, False)

    def print_profiler_summary(self):
        _check(_lib.xpbd_print_profiler_summary(self._h))

    # ---- extensions (no counterpart in the reference) ---------------------------
    def get_status(self):
        """(error_bits, lookback_timeouts, stack_overflows, slot_overflows) of the last step."""
        out = (C.c_uint32 * 4)()
        _check(_lib.xpbd_get_status(self._h, out))
        return tuple(int(x) for x in out)

    def step_async(self, dt=1.0 / 60.0, substeps=1, iterations=2):
        """Queue one frame on the solver's stream and return without waiting."""
        _check(_lib.xpbd_step_async(self._h, float(dt), int(substeps), int(iterations)))

    def sync(self):
        """Wait for queued frames, update last_contact_count and raise on a device error."""
        _check(_lib.xpbd_sync(self._h))

    @property
    def cuda_stream(self) -> int:
        """The solver's cudaStream_t as an integer handle (e.g. for torch.cuda.ExternalStream)."""
        return int(_lib.xpbd_stream(self._h) or 0)

    def set_profiling(self, on: bool):
        _check(_lib.xpbd_set_profiling(self._h, 1 if on else 0))

    def get_stage_times(self):
        """({stage name: accumulated device ms}, substeps) of synchronous profiled steps."""
        ms = (C.c_double * 32)()
        k = C.c_size_t(0)
        subs = C.c_uint64(0)
        _check(_lib.xpbd_get_stage_times(self._h, ms, 32, C.byref(k), C.byref(subs)))
        names = [_lib.xpbd_stage_name(i).decode() for i in range(k.value)]
        return {names[i]: float(ms[i]) for i in range(k.value)}, int(subs.value)

    def reset_stage_times(self):
        _check(_lib.xpbd_reset_stage_times(self._h))

    @property
    def kernels_launched(self):
        """Kernels launched by all frames run so far (xpbd_get_kernels_launched)."""
        v = C.c_uint64(0)
        _check(_lib.xpbd_get_kernels_launched(self._h, C.byref(v)))
        return int(v.value)

    def get_frame_stats(self):
        """{kernels, memsets} per frame of the last launched graph, frames run, cached graphs."""
        out = (C.c_uint64 * 4)()
        _check(_lib.xpbd_get_frame_stats(self._h, out))
        return {"kernels_per_frame": int(out[0]), "memsets_per_frame": int(out[1]), "frames": int(out[2]),
                "graphs": int(out[3])}
