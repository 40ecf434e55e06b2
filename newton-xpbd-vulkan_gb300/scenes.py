"""Seeded synthetic scenes with the shapes of the benchmark workloads.

The particle lattice follows the reference add-on's recipe
(latest_prebuilt/addons/newton_vulkan_plugin.py:363-374: meshgrid lattice,
centred, uniform jitter); Z is up as in the reference (plane z = altitude,
gravity (0, 0, -9.81)). No dataset is involved: every array is generated from
a fixed numpy seed so both the CUDA path and the CPU oracle see the same input.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

SEED_JITTER = 42
SEED_VELOCITY = 43
SEED_HEIGHTFIELD = 44
SEED_BOXES = 45
SEED_BATCH = 46
SEED_TARGET = 47


def lattice(dims, spacing, bottom_z, jitter, seed=SEED_JITTER, center_xy=(0.0, 0.0)):
    """dims=(nx, ny, nz) lattice, centred in x/y, lowest layer at bottom_z,
    jitter uniform in [-jitter, +jitter] per component."""
    nx, ny, nz = dims
    px = np.arange(nx) * spacing
    py = np.arange(ny) * spacing
    pz = np.arange(nz) * spacing
    pts = np.stack(np.meshgrid(px, py, pz)).reshape(3, -1).T
    ext = np.array([nx - 1, ny - 1, nz - 1], dtype=np.float64) * spacing
    pts = pts - np.array([ext[0] * 0.5, ext[1] * 0.5, 0.0])
    pts = pts + np.array([center_xy[0], center_xy[1], bottom_z])
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        pts = pts + (rng.random(pts.shape) - 0.5) * 2.0 * jitter
    return np.ascontiguousarray(pts, dtype=np.float32)


def heightfield(nv=256, extent=1.0, amplitude=0.025, waves=4, seed=SEED_HEIGHTFIELD):
    """nv x nv vertex grid over [-extent/2, extent/2]^2 with
    z = sum_k amplitude*sin(2*pi*k*(x cos t_k + y sin t_k) + p_k), k=1..waves;
    2*(nv-1)^2 triangles (130,050 for nv=256). Returns (verts[nv*nv,3], tris[T,3])."""
    rng = np.random.default_rng(seed)
    theta = rng.random(waves) * 2.0 * math.pi
    phase = rng.random(waves) * 2.0 * math.pi
    xs = np.linspace(-extent * 0.5, extent * 0.5, nv)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    Z = np.zeros_like(X)
    for k in range(waves):
        Z += amplitude * np.sin(2.0 * math.pi * (k + 1) * (X * math.cos(theta[k]) + Y * math.sin(theta[k])) + phase[k])
    verts = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1).astype(np.float32)
    i = np.arange(nv - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    v00 = (J * nv + I).ravel()
    v10 = v00 + 1
    v01 = v00 + nv
    v11 = v01 + 1
    tris = np.empty((v00.size * 2, 3), np.uint32)
    tris[0::2] = np.stack([v00, v10, v11], axis=1)
    tris[1::2] = np.stack([v00, v11, v01], axis=1)
    return verts, tris


def box_mesh(half_extents, center=(0.0, 0.0, 0.0), quat_xyzw=(0.0, 0.0, 0.0, 1.0)):
    """Closed 12-triangle box (outward winding), transformed to world space."""
    hx, hy, hz = half_extents
    c = np.array([[-1, -1, -1], [1, -1, -1], [1, 1, -1], [-1, 1, -1],
                  [-1, -1, 1], [1, -1, 1], [1, 1, 1], [-1, 1, 1]], np.float64)
    v = c * np.array([hx, hy, hz])
    x, y, z, w = quat_xyzw
    R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    v = v @ R.T + np.asarray(center, np.float64)
    t = np.array([[0, 2, 1], [0, 3, 2], [4, 5, 6], [4, 6, 7], [0, 1, 5], [0, 5, 4],
                  [2, 3, 7], [2, 7, 6], [1, 2, 6], [1, 6, 5], [3, 0, 4], [3, 4, 7]], np.uint32)
    return v.astype(np.float32), t


def box_inertia(half_extents, density=1000.0):
    """Mass and body-frame inertia tensor of a solid box."""
    hx, hy, hz = (float(h) for h in half_extents)
    m = density * 8.0 * hx * hy * hz
    inertia = np.diag([m / 3.0 * (hy * hy + hz * hz), m / 3.0 * (hx * hx + hz * hz), m / 3.0 * (hx * hx + hy * hy)])
    return m, inertia


def random_quats(n, rng):
    """Quaternions (xyzw) uniform on SO(3): normalised Gaussian 4-vectors."""
    q = rng.normal(size=(n, 4))
    return q / np.linalg.norm(q, axis=1, keepdims=True)


@dataclass
class Bodies:
    """Rigid-body table, one body per mesh (body b belongs to mesh b)."""
    q: np.ndarray            # (nb, 7) position xyz, quaternion xyzw
    qd: np.ndarray           # (nb, 6) linear, angular velocity
    com: np.ndarray          # (nb, 3)
    inertia: np.ndarray      # (nb, 3, 3)
    inv_inertia: np.ndarray  # (nb, 3, 3)
    inv_mass: np.ndarray     # (nb,)
    flags: np.ndarray        # (nb,)

    @staticmethod
    def static(nb):
        q = np.zeros((nb, 7), np.float32)
        q[:, 6] = 1.0
        z3 = np.zeros((nb, 3, 3), np.float32)
        return Bodies(q, np.zeros((nb, 6), np.float32), np.zeros((nb, 3), np.float32), z3.copy(), z3.copy(),
                      np.zeros(nb, np.float32), np.zeros(nb, np.int32))

    def set_box(self, b, half_extents, pos, quat_xyzw, density=1000.0, vel=(0, 0, 0), ang=(0, 0, 0)):
        m, inertia = box_inertia(half_extents, density)
        self.q[b, 0:3] = pos
        self.q[b, 3:7] = quat_xyzw
        self.qd[b, 0:3] = vel
        self.qd[b, 3:6] = ang
        self.inertia[b] = inertia
        self.inv_inertia[b] = np.linalg.inv(inertia)
        self.inv_mass[b] = 1.0 / m


@dataclass
class Scene:
    name: str
    config: dict
    positions: np.ndarray
    velocities: np.ndarray
    inv_mass: np.ndarray
    radii: np.ndarray
    flags: np.ndarray
    meshes: list = field(default_factory=list)  # (verts, tris, margin, watertight or None)
    bodies: object = None                        # Bodies for the meshes, or None (all static)
    dt: float = 1.0 / 60.0
    substeps: int = 10
    iterations: int = 1
    frames: int = 1

    @property
    def n(self) -> int:
        return int(self.positions.shape[0])

    def apply_config(self, cfg) -> None:
        for k, v in self.config.items():
            setattr(cfg, k, v)


def _base_config(radius, search_radius):
    return dict(
        soft_contact_mu=0.5, shape_material_mu=0.5, particle_mu=0.5,
        soft_contact_relaxation=0.9, particle_adhesion=0.0, particle_cohesion=0.0,
        particle_max_radius=radius, search_radius=search_radius, soft_contact_margin=0.01,
        enable_restitution=True, soft_contact_restitution=0.2, has_ground_plane=True,
        ground_plane_altitude=0.0, gravity=[0.0, 0.0, -9.81], particle_v_max=1e5,
    )


def pile(dims=(16, 16, 16), spacing=0.02, radius=0.01, jitter=0.002, bottom_z=0.02,
         inv_mass=1000.0, seed=SEED_JITTER, frames=120, name="pile") -> Scene:
    """Plain particle pile on the ground plane (4,096 particles for the default dims)."""
    x = lattice(dims, spacing, bottom_z, jitter, seed)
    n = x.shape[0]
    return Scene(name=name, config=_base_config(radius, 2.0 * radius), positions=x,
                 velocities=np.zeros_like(x), inv_mass=np.full(n, inv_mass, np.float32),
                 radii=np.full(n, radius, np.float32), flags=np.ones(n, np.int32), frames=frames)


def particles_on_mesh(dims=(64, 64, 64), spacing=0.01, radius=0.005, jitter=0.001, bottom_z=0.15,
                      hf_vertices=256, inv_mass=1000.0, frames=300, name="particles_on_mesh") -> Scene:
    """Lattice falling onto a sum-of-sines heightfield (262,144 particles, 130,050
    triangles for the defaults) with plane, mesh and particle-particle contacts."""
    sc = pile(dims, spacing, radius, jitter, bottom_z, inv_mass, frames=frames, name=name)
    v, t = heightfield(hf_vertices)
    sc.meshes.append((v, t, 0.0, None))
    return sc


def scaled(scene_fn, scale: int, **kw) -> Scene:
    """Same recipe with every lattice dimension divided by `scale` (test sizes)."""
    return scene_fn(**kw)


def pile_of(n, spacing=0.02, radius=0.01, jitter=0.002, bottom_z=0.02, inv_mass=1000.0,
            seed=SEED_JITTER, frames=100, name="pile") -> Scene:
    """Config-1-style pile of exactly n particles: a square-based lattice with side
    ceil(cbrt(n)), filled layer by layer from the bottom, the top layer partial."""
    side = max(1, int(math.ceil(round(n ** (1.0 / 3.0), 9))))
    layers = max(1, -(-n // (side * side)))
    x = lattice((side, side, layers), spacing, bottom_z, 0.0)
    order = np.argsort(x[:, 2], kind="stable")[:n]
    x = x[np.sort(order)]
    if jitter > 0.0:
        rng = np.random.default_rng(seed)
        x = (x + (rng.random(x.shape) - 0.5) * 2.0 * jitter).astype(np.float32)
    return Scene(name=name, config=_base_config(radius, 2.0 * radius), positions=np.ascontiguousarray(x),
                 velocities=np.zeros_like(x), inv_mass=np.full(n, inv_mass, np.float32),
                 radii=np.full(n, radius, np.float32), flags=np.ones(n, np.int32), frames=frames)


def batch_counts(n_scenes=512, lo=1024, hi=65536, seed=SEED_BATCH):
    """Per-scene particle counts log-uniform in [lo, hi]: round(exp(U[ln lo, ln hi]))."""
    rng = np.random.default_rng(seed)
    return [int(round(math.exp(u))) for u in rng.uniform(math.log(lo), math.log(hi), n_scenes)]


@dataclass
class Batch:
    """Independent scenes stepped by one batched solver (same configuration for all)."""
    scenes: list

    @property
    def counts(self):
        return [s.n for s in self.scenes]

    @property
    def n(self) -> int:
        return int(sum(self.counts))

    @property
    def config(self) -> dict:
        return self.scenes[0].config

    def apply_config(self, cfg) -> None:
        self.scenes[0].apply_config(cfg)

    def concat(self, attr):
        return np.ascontiguousarray(np.concatenate([getattr(s, attr) for s in self.scenes]))


def batch_bodies(batch: "Batch", shared: int = 1):
    """Meshes, body table and body scenes of one batched solver for scenes that each list
    the same `shared` static meshes first and then their own meshes: the shared meshes
    once (scene -1), then every scene's own meshes in scene order (scene s).
    Returns (meshes, Bodies, scene_of_body)."""
    first = batch.scenes[0]
    meshes = list(first.meshes[:shared])
    rows = [(first.bodies, b) for b in range(shared)]
    scene_of_body = [-1] * shared
    for s, sc in enumerate(batch.scenes):
        for b in range(shared, len(sc.meshes)):
            meshes.append(sc.meshes[b])
            rows.append((sc.bodies, b))
            scene_of_body.append(s)
    nb = len(meshes)
    out = Bodies.static(nb)
    for k, (src, b) in enumerate(rows):
        for name in ("q", "qd", "com", "inertia", "inv_inertia", "inv_mass", "flags"):
            getattr(out, name)[k] = getattr(src, name)[b]
    return meshes, out, np.array(scene_of_body, np.int32)


def batched_piles_with_boxes(n_scenes=512, lo=1024, hi=65536, max_boxes=16, seed=SEED_BATCH,
                             frames=100) -> Batch:
    """The batched piles with 0..max_boxes dynamic boxes per scene (uniform integer count,
    half-extents U[0.02, 0.08], density 1000, orientations uniform on SO(3), dropped in a
    column above the pile; seed + s per scene). Every scene lists the same static anchor
    mesh first (a small box far below the plane) so that mesh 0 is common to all scenes."""
    av, at = box_mesh((0.05, 0.05, 0.05), center=(0.0, 0.0, -10.0))
    counts = batch_counts(n_scenes, lo, hi, seed)
    out = []
    for s, c in enumerate(counts):
        rng = np.random.default_rng(seed + s)
        sc = pile_of(c, seed=seed + s, frames=frames, name=f"pile{s}")
        sc.meshes.append((av, at, 0.0, True))
        top = float(sc.positions[:, 2].max()) if c else 0.0
        nb = int(rng.integers(0, max_boxes + 1))
        he = rng.uniform(0.02, 0.08, (nb, 3)).astype(np.float32)
        xy = (rng.random((nb, 2)) - 0.5) * 0.1
        pos = [(float(xy[k, 0]), float(xy[k, 1]), top + 0.2 + 0.2 * k) for k in range(nb)]
        out.append(add_boxes(sc, [tuple(h) for h in he], pos, random_quats(nb, rng)))
    return Batch(out)


def batched_piles(n_scenes=512, lo=1024, hi=65536, seed=SEED_BATCH, frames=100) -> Batch:
    """Batched uneven scenes: n_scenes piles with log-uniform particle counts, scene s
    jittered with seed `seed + s`; plane only."""
    counts = batch_counts(n_scenes, lo, hi, seed)
    return Batch([pile_of(c, seed=seed + s, frames=frames, name=f"pile{s}") for s, c in enumerate(counts)])


def add_boxes(sc: Scene, half_extents, positions, quats, density=1000.0) -> Scene:
    """Appends one dynamic box body (a watertight 12-triangle mesh in its body frame) per row."""
    nb0 = len(sc.meshes)
    for he in half_extents:
        v, t = box_mesh(he)
        sc.meshes.append((v, t, 0.0, True))
    old = sc.bodies if sc.bodies is not None else Bodies.static(nb0)
    b = Bodies.static(len(sc.meshes))
    for name in ("q", "qd", "com", "inertia", "inv_inertia", "inv_mass", "flags"):
        getattr(b, name)[:nb0] = getattr(old, name)[:nb0]
    for k, (he, p, q) in enumerate(zip(half_extents, positions, quats)):
        b.set_box(nb0 + k, he, p, q, density)
    sc.bodies = b
    return sc


def mixed(dims=(128, 128, 64), spacing=0.01, radius=0.005, jitter=0.001, bottom_z=0.15, n_boxes=1024,
          hf_vertices=256, seed=SEED_BOXES, frames=200, name="mixed") -> Scene:
    """Particles, the heightfield and dynamic boxes: a dims lattice (1,048,576 particles for the
    defaults) on the plane and the sum-of-sines heightfield, plus n_boxes boxes with half-extents
    uniform in [0.02, 0.08] per axis, density 1000, orientations uniform on SO(3) and positions
    uniform over the lattice footprint, in a layer from 0.1 m to 1.1 m above its top."""
    sc = particles_on_mesh(dims, spacing, radius, jitter, bottom_z, hf_vertices, frames=frames, name=name)
    rng = np.random.default_rng(seed)
    he = rng.uniform(0.02, 0.08, size=(n_boxes, 3))
    quats = random_quats(n_boxes, rng)
    half_w = np.array([(dims[0] - 1) * spacing * 0.5, (dims[1] - 1) * spacing * 0.5])
    top = bottom_z + (dims[2] - 1) * spacing
    pos = np.empty((n_boxes, 3))
    pos[:, 0:2] = rng.uniform(-half_w, half_w, size=(n_boxes, 2))
    pos[:, 2] = rng.uniform(top + 0.1, top + 1.1, size=n_boxes)
    return add_boxes(sc, he, pos, quats)


def throw(dims=(32, 32, 32), spacing=0.02, radius=0.01, jitter=0.002, bottom_z=0.1, v_mean=(2.0, 3.0, 0.0),
          v_std=0.1, inv_mass=1000.0, seed=SEED_VELOCITY, frames=60, name="throw") -> Scene:
    """Differentiable throw: a dims lattice (32,768 particles for the defaults) with per-particle
    velocities ~ N(v_mean, v_std^2) per component (seed 43), falling from bottom_z onto the
    plane; plane and particle-particle contacts, restitution on."""
    sc = pile(dims, spacing, radius, jitter, bottom_z, inv_mass, frames=frames, name=name)
    rng = np.random.default_rng(seed)
    sc.velocities = (np.asarray(v_mean, np.float64) + v_std * rng.normal(size=(sc.n, 3))).astype(np.float32)
    return sc


def throw_target(seed=SEED_TARGET):
    """Target centroid of the throw loss: uniform in [-1, 1]^2 x [0, 0.5] (seed 47)."""
    rng = np.random.default_rng(seed)
    return np.array([rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(0, 0.5)], np.float64)
