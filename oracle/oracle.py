"""ctypes wrapper around the CPU oracle (test infrastructure only).

Loaded by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg to
check or time the CUDA path; never imported by the product package.
`build()` compiles oracle/_build/liboracle_{f32,f64}.so with the Makefile next
to this file (and oracle/_ref/libref_bvh.so when the reference checkout exists).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REFDIR = os.path.join(HERE, "_ref")
NUM_CELLS = 128 ** 3


def reference_checkout():
    """The reference checkout the BVH shim is compiled from: $XPBD_REFERENCE_DIR, else the
    build container's checkout; None where neither exists (the GPU machine has none)."""
    for d in (os.environ.get("XPBD_REFERENCE_DIR"), "/root/reference"):
        if d and os.path.exists(os.path.join(d, "src", "mesh_bvh.h")):
            return d
    return None


def build() -> None:
    """Oracle libraries, plus the reference's BVH shim where the checkout exists (Makefile REF)."""
    subprocess.check_call(["make", "-s", "-C", HERE, "-j2", "all"])
    ref = reference_checkout()
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref-if-present", f"REF={ref}"])


class Config(C.Structure):
    """Mirrors vkx::SolverConfig's numeric fields (src/scene.h:14-41)."""

    _fields_ = [
        ("dt", C.c_float), ("substeps", C.c_int32), ("iterations", C.c_int32),
        ("particle_v_max", C.c_float), ("soft_contact_mu", C.c_float),
        ("shape_material_mu", C.c_float), ("soft_contact_relaxation", C.c_float),
        ("particle_adhesion", C.c_float), ("particle_mu", C.c_float),
        ("particle_cohesion", C.c_float), ("particle_max_radius", C.c_float),
        ("search_radius", C.c_float), ("soft_contact_margin", C.c_float),
        ("enable_restitution", C.c_int32), ("soft_contact_restitution", C.c_float),
        ("has_ground_plane", C.c_int32), ("ground_plane_altitude", C.c_float),
        ("gravity", C.c_float * 3),
    ]

    @classmethod
    def from_obj(cls, cfg) -> "Config":
        c = cls()
        for name, _ in cls._fields_:
            if name == "gravity":
                g = list(cfg.gravity)
                c.gravity[0], c.gravity[1], c.gravity[2] = g[0], g[1], g[2]
            else:
                setattr(c, name, getattr(cfg, name))
        return c


class SolverConfig:
    """vkx::SolverConfig's numeric fields with the reference's defaults (src/scene.h:15-40),
    as a plain object: the oracle's own configuration, built without the product library."""

    def __init__(self):
        self.dt = 1.0 / 60.0
        self.substeps = 1
        self.iterations = 2
        self.particle_v_max = 1e5
        self.soft_contact_mu = 0.5
        self.shape_material_mu = 1.0
        self.soft_contact_relaxation = 0.9
        self.particle_adhesion = 0.0
        self.particle_mu = 0.5
        self.particle_cohesion = 0.0
        self.particle_max_radius = 0.02
        self.search_radius = 0.04
        self.soft_contact_margin = 0.01
        self.enable_restitution = False
        self.soft_contact_restitution = 0.0
        self.has_ground_plane = True
        self.ground_plane_altitude = 0.0
        self.gravity = [0.0, 0.0, -9.81]


_P = C.c_void_p
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int32)
_U = C.POINTER(C.c_uint32)
class BodyParams(C.Structure):
    _fields_ = [("angular_damping", C.c_float), ("rigid_contact_margin", C.c_float),
                ("rigid_contact_relaxation", C.c_float), ("rigid_contact_con_weighting", C.c_int32),
                ("rigid_mu_torsional", C.c_float), ("rigid_mu_rolling", C.c_float),
                ("particle_contact_con_weighting", C.c_int32)]


BODY_PARAM_DEFAULTS = dict(angular_damping=0.0, rigid_contact_margin=0.01, rigid_contact_relaxation=0.8,
                           rigid_contact_con_weighting=1, rigid_mu_torsional=0.0, rigid_mu_rolling=0.0,
                           particle_contact_con_weighting=1)

_libs: dict = {}


def _fp(a, t):
    return None if a is None else a.ctypes.data_as(t)


def load(precision: str = "f32") -> C.CDLL:
    if precision in _libs:
        return _libs[precision]
    path = os.path.join(BUILD, f"liboracle_{precision}.so")
    if not os.path.exists(path):
        build()
    lib = C.CDLL(path)
    lib.or_create.restype = _P
    lib.or_create.argtypes = [C.POINTER(Config), C.c_int64, C.c_int64]
    lib.or_destroy.argtypes = [_P]
    lib.or_add_mesh.argtypes = [_P, _F, C.c_int64, _U, C.c_int64, C.c_float, _F, C.c_int]
    lib.or_finalize_meshes.argtypes = [_P]
    lib.or_update_mesh.argtypes = [_P, C.c_int64, _F, C.c_int64, _F]
    lib.or_set_particles.argtypes = [_P, _F, _F, _F, _F, _I, C.c_int64]
    lib.or_set_bodies.argtypes = [_P, _F, _F, _F, _F, _F, _F, _I, C.c_int64]
    lib.or_get_bodies.argtypes = [_P, _F, _F]
    lib.or_set_body_params.argtypes = [_P, C.POINTER(BodyParams)]
    _DP = C.POINTER(C.c_double)
    lib.or_rollout.argtypes = [_P, C.c_float, C.c_int, C.c_int, C.c_int]
    lib.or_rollout_backward.argtypes = [_P, _F, _F, _DP, _DP, _DP, _DP]
    lib.or_rigid_contact_overflows.restype = C.c_int64
    lib.or_rigid_contact_overflows.argtypes = [_P]
    lib.or_step.argtypes = [_P, C.c_float, C.c_int, C.c_int]
    lib.or_collide_only.argtypes = [_P]
    lib.or_step_solve_only.argtypes = [_P, C.c_float, C.c_int, C.c_int]
    lib.or_set_contact_data.argtypes = [_P, _I, _I, _F, _F, C.c_int64]
    lib.or_get_positions.argtypes = [_P, _F]
    lib.or_get_velocities.argtypes = [_P, _F]
    lib.or_get_state64.argtypes = [_P, _D, _D]
    lib.or_contact_count.restype = C.c_int64
    lib.or_contact_count.argtypes = [_P]
    lib.or_contact_count_raw.restype = C.c_int64
    lib.or_contact_count_raw.argtypes = [_P]
    lib.or_get_contacts.argtypes = [_P, _I, _I, _F, _F, _F]
    lib.or_get_sorted.argtypes = [_P, _U, _U]
    lib.or_get_cell_starts.argtypes = [_P, _I]
    lib.or_get_cell_ends.argtypes = [_P, _I]
    lib.or_get_deltas.argtypes = [_P, _F]
    lib.or_mesh_bvh_node_count.restype = C.c_int64
    lib.or_mesh_bvh_node_count.argtypes = [_P, C.c_int64]
    lib.or_get_mesh_bvh.argtypes = [_P, C.c_int64, _F, _F]
    lib.or_mesh_is_watertight_flag.argtypes = [_P, C.c_int64]
    lib.or_mesh_avg_edge.restype = C.c_float
    lib.or_mesh_avg_edge.argtypes = [_P, C.c_int64]
    lib.or_bvh_build.argtypes = [_F, C.c_int64, _U, C.c_int64, _F, _F, _U, _U]
    lib.or_bvh_refit.argtypes = [_F, _U, _F, _F, _U, C.c_uint32]
    lib.or_tris_watertight.argtypes = [_U, C.c_int64, C.c_int64]
    lib.or_closest_point_triangle.argtypes = [_F, _F, _F, _F, _F, _F, _F]
    lib.or_acos.restype = C.c_float
    lib.or_acos.argtypes = [C.c_float]
    lib.or_set_threads.argtypes = [C.c_int]
    lib.or_get_threads.restype = C.c_int
    _libs[precision] = lib
    return lib


def f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def u32(a):
    return np.ascontiguousarray(a, dtype=np.uint32)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


class OracleSolver:
    """Same call surface as vkxpbd.XpbdSolver, executed by the C oracle."""

    def __init__(self, cfg, num_particles: int, max_contacts: int = 0, precision: str = "f32"):
        self.lib = load(precision)
        self._cfg = Config.from_obj(cfg)
        self.n = int(num_particles)
        self.h = self.lib.or_create(C.byref(self._cfg), self.n, int(max_contacts))
        self.cmax = int(max_contacts) if max_contacts else 2 * self.n
        self.meshes = 0

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            self.lib.or_destroy(h)
            self.h = None

    def add_mesh(self, vertices, indices, shape_margin=0.0, shape_rot=None, is_watertight=None):
        v, t = f32(vertices).reshape(-1), u32(indices).reshape(-1)
        rot = None if shape_rot is None else f32(shape_rot)
        wt = -1 if is_watertight is None else int(bool(is_watertight))
        self.lib.or_add_mesh(self.h, _fp(v, _F), v.size // 3, _fp(t, _U), t.size // 3,
                             float(shape_margin), _fp(rot, _F), wt)
        self.meshes += 1

    def finalize_meshes(self):
        self.lib.or_finalize_meshes(self.h)

    def update_mesh(self, mesh_index, verts, velocities=None):
        v = f32(verts).reshape(-1)
        vel = None if velocities is None else f32(velocities).reshape(-1)
        rc = self.lib.or_update_mesh(self.h, int(mesh_index), _fp(v, _F), v.size // 3, _fp(vel, _F))
        if rc != 0:
            raise RuntimeError(f"oracle update_mesh failed ({rc})")

    def set_particles(self, q, qd=None, inv_mass=None, radii=None, flags=None):
        q = f32(q).reshape(-1)
        qd = None if qd is None else f32(qd).reshape(-1)
        w = None if inv_mass is None else f32(inv_mass)
        r = None if radii is None else f32(radii)
        fl = None if flags is None else i32(flags)
        rc = self.lib.or_set_particles(self.h, _fp(q, _F), _fp(qd, _F), _fp(w, _F), _fp(r, _F),
                                       _fp(fl, _I), q.size // 3)
        if rc != 0:
            raise RuntimeError("Particle count mismatch")

    def set_bodies(self, q=None, qd=None, com=None, inertia=None, inv_inertia=None, inv_mass=None, flags=None):
        """q: (nb, 7) position xyz + quaternion xyzw; qd: (nb, 6) linear, angular velocity;
        com (nb, 3); inertia, inv_inertia (nb, 3, 3); inv_mass (nb,); flags (nb,)."""
        nb = self.meshes
        q8 = qd8 = None
        if q is not None:
            q = f32(q).reshape(nb, 7)
            q8 = np.zeros((nb, 8), np.float32)
            q8[:, 0:3] = q[:, 0:3]
            q8[:, 4:8] = q[:, 3:7]
        if qd is not None:
            qd = f32(qd).reshape(nb, 6)
            qd8 = np.zeros((nb, 8), np.float32)
            qd8[:, 0:3] = qd[:, 0:3]
            qd8[:, 4:7] = qd[:, 3:6]
        arrs = [None if a is None else f32(a).reshape(-1) for a in (q8, qd8, com, inertia, inv_inertia, inv_mass)]
        fl = None if flags is None else i32(flags)
        rc = self.lib.or_set_bodies(self.h, *[_fp(a, _F) for a in arrs], _fp(fl, _I), nb)
        if rc != 0:
            raise RuntimeError("oracle set_bodies failed")

    def get_body_q(self):
        q8 = np.zeros((self.meshes, 8), np.float32)
        self.lib.or_get_bodies(self.h, _fp(q8, _F), None)
        return np.ascontiguousarray(np.concatenate([q8[:, 0:3], q8[:, 4:8]], axis=1))

    def get_body_qd(self):
        qd8 = np.zeros((self.meshes, 8), np.float32)
        self.lib.or_get_bodies(self.h, None, _fp(qd8, _F))
        return np.ascontiguousarray(np.concatenate([qd8[:, 0:3], qd8[:, 4:7]], axis=1))

    def set_body_params(self, **kw):
        bp = BodyParams()
        for k, v in {**BODY_PARAM_DEFAULTS, **kw}.items():
            setattr(bp, k, v)
        self.lib.or_set_body_params(self.h, C.byref(bp))

    def rollout(self, dt, substeps, frames, iterations=1):
        rc = self.lib.or_rollout(self.h, float(dt), int(substeps), int(iterations), int(frames))
        if rc != 0:
            raise RuntimeError("oracle rollout: plane and particle contacts only, one iteration")

    def rollout_backward(self, gx_final, gv_final=None):
        """Adjoint of the last rollout: dict of gradients (float64) w.r.t. initial positions,
        initial velocities, inverse masses and the contact parameters."""
        n = self.n
        gx = f32(gx_final).reshape(-1)
        gv = None if gv_final is None else f32(gv_final).reshape(-1)
        out = {k: np.zeros(sz, np.float64) for k, sz in (("x0", 3 * n), ("v0", 3 * n), ("inv_mass", n), ("params", 4))}
        D = C.POINTER(C.c_double)
        rc = self.lib.or_rollout_backward(self.h, _fp(gx, _F), _fp(gv, _F), out["x0"].ctypes.data_as(D),
                                          out["v0"].ctypes.data_as(D), out["inv_mass"].ctypes.data_as(D),
                                          out["params"].ctypes.data_as(D))
        if rc == -2:
            raise RuntimeError("oracle rollout_backward: the v_max clamp fired in the forward pass")
        if rc != 0:
            raise RuntimeError("oracle rollout_backward: no rollout")
        out["x0"] = out["x0"].reshape(n, 3)
        out["v0"] = out["v0"].reshape(n, 3)
        p = out.pop("params")
        out.update(soft_contact_mu=p[0], shape_material_mu=p[1], particle_mu=p[2], soft_contact_restitution=p[3])
        return out

    def rigid_contact_overflows(self):
        return int(self.lib.or_rigid_contact_overflows(self.h))

    def step(self, dt=1.0 / 60.0, substeps=1, iterations=2):
        self.lib.or_step(self.h, float(dt), int(substeps), int(iterations))

    def collide_only(self):
        self.lib.or_collide_only(self.h)

    def step_solve_only(self, dt, substeps, iterations):
        self.lib.or_step_solve_only(self.h, float(dt), int(substeps), int(iterations))

    def set_contact_data(self, particles, shapes, body_positions, normals, contact_count):
        p, s = i32(particles), i32(shapes)
        bp, nn = f32(body_positions).reshape(-1), f32(normals).reshape(-1)
        self.lib.or_set_contact_data(self.h, _fp(p, _I), _fp(s, _I), _fp(bp, _F), _fp(nn, _F),
                                     int(contact_count))

    def get_positions(self):
        out = np.empty((self.n, 3), np.float32)
        self.lib.or_get_positions(self.h, _fp(out, _F))
        return out

    def get_velocities(self):
        out = np.empty((self.n, 3), np.float32)
        self.lib.or_get_velocities(self.h, _fp(out, _F))
        return out

    def get_state64(self):
        x = np.empty((self.n, 3), np.float64)
        v = np.empty((self.n, 3), np.float64)
        self.lib.or_get_state64(self.h, _fp(x, _D), _fp(v, _D))
        return x, v

    @property
    def last_contact_count(self):
        return int(self.lib.or_contact_count(self.h))

    @property
    def raw_contact_count(self):
        return int(self.lib.or_contact_count_raw(self.h))

    def get_contacts(self):
        m = self.last_contact_count
        p = np.empty(m, np.int32)
        s = np.empty(m, np.int32)
        bp = np.empty((m, 3), np.float32)
        bv = np.empty((m, 3), np.float32)
        nn = np.empty((m, 3), np.float32)
        self.lib.or_get_contacts(self.h, _fp(p, _I), _fp(s, _I), _fp(bp, _F), _fp(bv, _F), _fp(nn, _F))
        return {"particles": p, "shapes": s, "body_positions": bp, "body_velocities": bv, "normals": nn}

    def get_sorted(self):
        c = np.empty(self.n, np.uint32)
        i = np.empty(self.n, np.uint32)
        self.lib.or_get_sorted(self.h, _fp(c, _U), _fp(i, _U))
        return c, i

    def get_cell_starts(self):
        out = np.empty(NUM_CELLS, np.int32)
        self.lib.or_get_cell_starts(self.h, _fp(out, _I))
        return out

    def get_cell_ends(self):
        out = np.empty(NUM_CELLS, np.int32)
        self.lib.or_get_cell_ends(self.h, _fp(out, _I))
        return out

    def get_deltas(self):
        out = np.empty((self.n, 3), np.float32)
        self.lib.or_get_deltas(self.h, _fp(out, _F))
        return out

    def get_mesh_bvh(self, i):
        k = int(self.lib.or_mesh_bvh_node_count(self.h, i))
        lo = np.empty((k, 4), np.float32)
        hi = np.empty((k, 4), np.float32)
        self.lib.or_get_mesh_bvh(self.h, i, _fp(lo, _F), _fp(hi, _F))
        return lo, hi

    def mesh_watertight(self, i):
        return bool(self.lib.or_mesh_is_watertight_flag(self.h, i))

    def mesh_avg_edge(self, i):
        return float(self.lib.or_mesh_avg_edge(self.h, i))


def bvh_build(pts, tris, precision="f32"):
    """LBVH of one mesh: (lowers[2T,4], uppers[2T,4], prims[T], root)."""
    lib = load(precision)
    p, t = f32(pts).reshape(-1), u32(tris).reshape(-1)
    nt = t.size // 3
    lo = np.zeros((2 * nt, 4), np.float32)
    hi = np.zeros((2 * nt, 4), np.float32)
    pr = np.zeros(nt, np.uint32)
    root = C.c_uint32(0)
    lib.or_bvh_build(_fp(p, _F), p.size // 3, _fp(t, _U), nt, _fp(lo, _F), _fp(hi, _F), _fp(pr, _U),
                     C.byref(root))
    return lo, hi, pr, int(root.value)


def bvh_refit(pts, tris, lowers, uppers, prims, root, precision="f32"):
    lib = load(precision)
    p, t = f32(pts).reshape(-1), u32(tris).reshape(-1)
    lo, hi = lowers.copy(), uppers.copy()
    lib.or_bvh_refit(_fp(p, _F), _fp(t, _U), _fp(lo, _F), _fp(hi, _F), _fp(u32(prims), _U), int(root))
    return lo, hi


def tris_watertight(tris, num_verts):
    lib = load("f32")
    t = u32(tris).reshape(-1)
    return bool(lib.or_tris_watertight(_fp(t, _U), t.size // 3, int(num_verts)))


def acos32(x: float) -> float:
    return float(load("f32").or_acos(float(x)))


# ---- the reference's own BVH code, compiled in place (only where the checkout exists) ----
def load_ref():
    path = os.path.join(REFDIR, "libref_bvh.so")
    if not os.path.exists(path):
        return None
    lib = C.CDLL(path)
    lib.ref_bvh_build.argtypes = [_F, C.c_int64, _U, C.c_int64, _F, _F, _U, _U]
    lib.ref_bvh_build_refit.argtypes = [_F, _F, C.c_int64, _U, C.c_int64, _F, _F]
    lib.ref_query_closest.argtypes = [_F, C.c_int64, _U, C.c_int64, _F, C.c_float, _U, _F]
    return lib


def ref_bvh_build(lib, pts, tris):
    p, t = f32(pts).reshape(-1), u32(tris).reshape(-1)
    nt = t.size // 3
    lo = np.zeros((2 * nt, 4), np.float32)
    hi = np.zeros((2 * nt, 4), np.float32)
    pr = np.zeros(nt, np.uint32)
    root = C.c_uint32(0)
    lib.ref_bvh_build(_fp(p, _F), p.size // 3, _fp(t, _U), nt, _fp(lo, _F), _fp(hi, _F), _fp(pr, _U),
                      C.byref(root))
    return lo, hi, pr, int(root.value)


def ref_bvh_build_refit(lib, pts, pts_new, tris):
    p, pn, t = f32(pts).reshape(-1), f32(pts_new).reshape(-1), u32(tris).reshape(-1)
    nt = t.size // 3
    lo = np.zeros((2 * nt, 4), np.float32)
    hi = np.zeros((2 * nt, 4), np.float32)
    lib.ref_bvh_build_refit(_fp(p, _F), _fp(pn, _F), p.size // 3, _fp(t, _U), nt, _fp(lo, _F), _fp(hi, _F))
    return lo, hi
