"""Seeded synthetic scenes (no dataset is involved anywhere on this path).

The five workloads follow the benchmark configurations of the project
(pyramid, cube field, mixed convex pile, 1024 batched joint scenes,
split-precision wall throw); the small scenes mirror the reference demos'
setups (demos/avbd_box, demos/constraints) and are used by the tests.
The ground plane is the floor of a large container box
(engine/src/physics/gpu.rs:352-404), the reference's only ground mechanism.
"""
from dataclasses import dataclass, field

import numpy as np

from . import abi
from . import physics as ph


@dataclass
class Scene:
    name: str
    bodies: np.ndarray
    state: np.ndarray
    constraints: np.ndarray = field(default_factory=lambda: np.zeros(0, abi.CONSTRAINT))
    scene_offsets: np.ndarray = None
    containers: list = None
    hull_vertices: np.ndarray = None
    options: object = None
    steps: int = 1
    positions_f64: np.ndarray = None

    @property
    def n(self):
        return len(self.bodies)

    @property
    def n_scenes(self):
        return 1 if self.scene_offsets is None else len(self.scene_offsets) - 1

    def split(self, groups):
        """Contiguous runs of whole scenes with about equal body counts, as
        separate Scenes (joints rebased; hull vertices shared).  Returns the
        Scenes and the body offset of each in this one."""
        off = np.array([0, self.n], np.int64) if self.scene_offsets is None else self.scene_offsets.astype(np.int64)
        ns = len(off) - 1
        groups = max(1, min(int(groups), ns))
        cuts = [0]
        for g in range(1, groups):
            s = int(np.searchsorted(off, self.n * g / groups))
            cuts.append(min(max(s, cuts[-1] + 1), ns - (groups - g)))
        cuts.append(ns)
        out, starts = [], []
        for g in range(groups):
            s0, s1 = cuts[g], cuts[g + 1]
            lo, hi = int(off[s0]), int(off[s1])
            c = self.constraints
            keep = (c["a"] >= lo) & (c["a"] < hi)
            c = c[keep].copy()
            c["a"] -= lo
            c["b"] -= lo
            sub = Scene(f"{self.name}[{s0}:{s1}]", self.bodies[lo:hi].copy(), self.state[lo:hi].copy(),
                        constraints=c, hull_vertices=self.hull_vertices, options=self.options, steps=self.steps,
                        positions_f64=None if self.positions_f64 is None else self.positions_f64[lo:hi].copy())
            if self.scene_offsets is not None:
                sub.scene_offsets = (off[s0:s1 + 1] - lo).astype(np.uint32)
            if self.containers is not None:
                sub.containers = self.containers[s0:s1] if self.scene_offsets is not None else self.containers
            out.append(sub)
            starts.append(lo)
        return out, starts

    def select(self, indices):
        """The scenes `indices` (in that order) as one packed Scene: bodies,
        containers and joints of each, joints rebased (hull vertices shared)."""
        off = np.array([0, self.n], np.int64) if self.scene_offsets is None else self.scene_offsets.astype(np.int64)
        idx = [int(i) for i in indices]
        c = self.constraints
        cs = np.searchsorted(off, c["a"].astype(np.int64), side="right") - 1 if len(c) else np.zeros(0, np.int64)
        bodies, states, cons, offs, conts = [], [], [], [0], []
        for s in idx:
            lo, hi = int(off[s]), int(off[s + 1])
            bodies.append(self.bodies[lo:hi])
            states.append(self.state[lo:hi])
            j = c[cs == s].copy()
            j["a"] = (j["a"].astype(np.int64) - lo + offs[-1]).astype(j["a"].dtype)
            j["b"] = (j["b"].astype(np.int64) - lo + offs[-1]).astype(j["b"].dtype)
            cons.append(j)
            offs.append(offs[-1] + hi - lo)
            if self.containers is not None:
                conts.append(self.containers[s] if self.scene_offsets is not None else self.containers[0])
        return Scene(f"{self.name}[{len(idx)} scenes]", np.concatenate(bodies) if bodies else self.bodies[:0].copy(),
                     np.concatenate(states) if states else self.state[:0].copy(),
                     constraints=np.concatenate(cons) if cons else c[:0].copy(),
                     scene_offsets=np.array(offs, np.uint32), containers=conts if self.containers is not None else None,
                     hull_vertices=self.hull_vertices, options=self.options, steps=self.steps)

    def upload_kwargs(self):
        return dict(constraints=self.constraints, scene_offsets=self.scene_offsets, containers=self.containers,
                    hull_vertices=self.hull_vertices, positions_f64=self.positions_f64)


def ground(height=1000.0, y0=0.0, x0=0.0):
    """A container whose floor is the plane y = y0 (walls far away)."""
    return ph.container((x0, y0 + height, 0.0), height)


def random_quats(rng, n):
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    return q.astype(np.float32)


def icosphere42():
    """Level-1 subdivided icosahedron: 12 + 30 unit vertices."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    v = [np.array(x, np.float64) / np.linalg.norm(x) for x in v]
    faces = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
             (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11),
             (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    mids = {}
    for f in faces:
        for a, b in ((f[0], f[1]), (f[1], f[2]), (f[2], f[0])):
            k = (min(a, b), max(a, b))
            if k not in mids:
                m = v[a] + v[b]
                mids[k] = m / np.linalg.norm(m)
    verts = np.array(v + [mids[k] for k in sorted(mids)], np.float64)
    assert len(verts) == 42
    return verts


def regular_tetrahedron(edge):
    c = np.array([(1, 1, 1), (1, -1, -1), (-1, 1, -1), (-1, -1, 1)], np.float64)
    return (c * (edge / (2.0 * 2 ** 0.5))).astype(np.float32)


# ------------------------------------------------------------ workloads
def pyramid(levels=10, side=1.0, gap=0.01, density=1000.0):
    """Plain AVBD box pyramid: `levels` rows of unit cubes (55 for 10 levels)
    with 0.01 m gaps on the ground; g = -9.81, dt = 1/60, 10 iterations,
    alpha 0.95, beta 1e5, k0 1e4, friction 0.5, 600 steps."""
    h = side / 2.0
    mass = density * side ** 3
    items = []
    for k in range(levels):
        count = levels - k
        y = h + gap + k * (side + gap)
        for i in range(count):
            x = (i - (count - 1) / 2.0) * (side + gap)
            items.append(ph.cube((x, y, 0.0), h, mass))
    b, s = ph.pack_bodies(items)
    o = ph.avbd_options(gravity=(0, -9.81, 0), alpha=0.95, beta_lin=1e5, penalty_min=1e4, friction=0.5,
                        iterations=10)
    return Scene(f"pyramid{len(b)}", b, s, containers=[ground()], options=o, steps=600)


def cube_field(nx=32, nz=32, ny=8, side=0.5, spacing=0.6, jitter=0.05, drop=2.0, density=1000.0, seed=2):
    """Cube field: nx x ny x nz cubes of side 0.5 on a 0.6 grid with +-0.05
    jitter and random orientations, dropped from y = 2; friction 0.6,
    dt = 1/60, 10 iterations, 300 steps."""
    rng = np.random.default_rng(0x5EED + seed)
    n = nx * ny * nz
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    pos = np.stack([(ix.ravel() - (nx - 1) / 2) * spacing, drop + iy.ravel() * spacing,
                    (iz.ravel() - (nz - 1) / 2) * spacing], 1)
    pos = pos + rng.uniform(-jitter, jitter, size=pos.shape)
    q = random_quats(rng, n)
    mass = density * side ** 3
    items = [ph.cube(pos[i], side / 2.0, mass, orientation=q[i]) for i in range(n)]
    b, s = ph.pack_bodies(items)
    o = ph.avbd_options(gravity=(0, -9.81, 0), friction=0.6, iterations=10)
    return Scene(f"cube_field{n}", b, s, containers=[ground()], options=o, steps=300)


def mixed_pile(n=50000, extent=40.0, seed=3):
    """Mixed convex pile: 40% boxes (lognormal half extents, mu ln 0.25,
    sigma 0.3), 40% 42-vertex icosphere hulls (lognormal radius), 20%
    tetrahedra (edge 0.4); uniform positions in a 40 m cube above the ground,
    density U(500, 2000); dt = 1/120, 12 iterations, 500 steps."""
    rng = np.random.default_rng(0x5EED + seed)
    ico = icosphere42()
    tet = regular_tetrahedron(0.4)
    kinds = rng.permutation(np.repeat([0, 1, 2], [int(0.4 * n), int(0.4 * n), n - 2 * int(0.4 * n)]))
    pos = np.stack([rng.uniform(-extent / 2, extent / 2, n), rng.uniform(1.0, 1.0 + extent, n),
                    rng.uniform(-extent / 2, extent / 2, n)], 1)
    q = random_quats(rng, n)
    rho = rng.uniform(500.0, 2000.0, n)
    hull = []
    items = []
    for i in range(n):
        if kinds[i] == 0:
            h = np.exp(rng.normal(np.log(0.25), 0.3, 3))
            items.append(ph.box(pos[i], h, rho[i] * 8 * h.prod(), orientation=q[i]))
        elif kinds[i] == 1:
            r = float(np.exp(rng.normal(np.log(0.25), 0.3)))
            verts = (ico * r).astype(np.float32)
            first = len(hull) * 42
            hull.append(verts)
            items.append(ph.hull(pos[i], first, verts, rho[i] * 4.0 / 3.0 * np.pi * r ** 3, orientation=q[i]))
        else:
            vol = 0.4 ** 3 / (6 * 2 ** 0.5)
            items.append(ph.tetrahedron(pos[i], tet, rho[i] * vol, orientation=q[i]))
    b, s = ph.pack_bodies(items)
    hv = np.zeros((len(hull) * 42, 4), np.float32)
    if hull:
        hv[:, :3] = np.concatenate(hull)
    o = ph.avbd_options(gravity=(0, -9.81, 0), dt=1.0 / 120.0, iterations=12)
    return Scene(f"mixed_pile{n}", b, s, containers=[ground()], hull_vertices=hv, options=o, steps=500)


def joint_scene(rng, n_bodies):
    """One scene of the batched workload: rope chains (max-distance rows,
    0.2 m links), ball-socket pendulum chains of length 2-20, Hookean springs
    (k = 1e3, rest 0.5) and 0-200 loose boxes on the ground."""
    items, joints = [], []
    n_loose = int(rng.integers(0, min(200, n_bodies // 2) + 1))
    budget = n_bodies - n_loose
    link_r = 0.05
    # chains hang from static anchors on a 2 m grid in x-z (all inside the
    # container, clear of each other's swing at rest)
    grid = int(np.ceil(np.sqrt(max(1, budget / 8.0))))
    slot = 0
    kind = 0
    while budget > 0:
        length = int(min(budget, rng.integers(2, 21)))
        base = len(items)
        x = (slot % grid - grid / 2.0) * 2.0
        z = (slot // grid - grid / 2.0) * 2.0
        slot += 1
        top = 12.0 + rng.uniform(0.0, 2.0)
        items.append(ph.sphere((x, top, z), link_r, 0.0))  # static anchor
        for k in range(1, length):
            if kind == 0:  # rope chain
                p = (x + 0.2 * k * 0.7, top - 0.2 * k * 0.7, z)
            elif kind == 1:  # pendulum
                p = (x + 0.2 * k, top, z)
            else:  # springs
                p = (x, top - 0.5 * k, z + 0.05 * k)
            items.append(ph.sphere(p, link_r, 1.0))
            a, b = base + k - 1, base + k
            if kind == 0:
                joints.append(ph.rope(a, b, (0, 0, 0), (0, 0, 0), 0.2))
            elif kind == 1:
                joints.append(ph.ball_socket(a, b, (0.1, 0, 0), (-0.1, 0, 0)))
            else:
                joints.append(ph.spring(a, b, (0, 0, 0), (0, 0, 0), 1e3, 0.5))
        budget -= length
        kind = (kind + 1) % 3
    # loose boxes on a 0.5 m grid beside the chain grid
    side = int(np.ceil(np.sqrt(max(n_loose, 1))))
    x0 = grid + 4.0
    for k in range(n_loose):
        i, j = k % side, k // side
        h = float(rng.uniform(0.1, 0.2))
        p = (x0 + i * 0.5 + rng.uniform(-0.02, 0.02), h + 0.02 + rng.uniform(0, 0.5), -4.0 + j * 0.5)
        items.append(ph.cube(p, h, 8 * h ** 3 * 1000.0))
    return items, joints


def batched(n_scenes=1024, lo=16, hi=2048, seed=4):
    """1024 independent scenes, body counts log-uniform in [16, 2048];
    dt = 1/60, 10 iterations, 600 steps."""
    rng = np.random.default_rng(0x5EED + seed)
    sizes = np.floor(np.exp(rng.uniform(np.log(lo), np.log(hi), n_scenes))).astype(int)
    all_items, all_joints, offsets = [], [], [0]
    for s in range(n_scenes):
        items, joints = joint_scene(rng, int(sizes[s]))
        base = len(all_items)
        for j in joints:
            j = j.copy()
            j["a"] += base
            j["b"] += base
            all_joints.append(j)
        all_items.extend(items)
        offsets.append(len(all_items))
    b, st = ph.pack_bodies(all_items)
    cons = ph.pack_joints(all_joints)
    o = ph.avbd_options(gravity=(0, -9.81, 0), iterations=10)
    return Scene(f"batched{n_scenes}", b, st, constraints=cons, scene_offsets=np.array(offsets, np.uint32),
                 containers=[ground(1000.0)] * n_scenes, options=o, steps=600)


def wall_throw(cols=400, rows=500, projectiles=1000, offset=1.0e5, seed=5):
    """Split-precision wall throw: a cols x rows wall of 0.4 x 0.2 x 0.2 m
    bricks (density 2000) at x = 1e5 m and spheres of radius 0.3 launched
    at 30 m/s with +-5 degree jitter; dt = 1/120, 15 iterations, 600 steps."""
    rng = np.random.default_rng(0x5EED + seed)
    items, pos64 = [], []
    he = (0.1, 0.1, 0.2)
    m = 0.4 * 0.2 * 0.2 * 2000.0
    for r in range(rows):
        for c in range(cols):
            z = (c - (cols - 1) / 2.0) * 0.4 + (0.2 if r % 2 else 0.0)
            p = (offset, 0.1 + r * 0.2, z)
            items.append(ph.box(p, he, m))
            pos64.append(p)
    for k in range(projectiles):
        yaw, pitch = np.radians(rng.uniform(-5, 5, 2))
        d = np.array([np.cos(pitch) * np.cos(yaw), np.sin(pitch), np.cos(pitch) * np.sin(yaw)])
        p = (offset - 15.0 - rng.uniform(0, 10), rng.uniform(1.0, rows * 0.2 * 0.8),
             rng.uniform(-cols * 0.15, cols * 0.15))
        items.append(ph.sphere(p, 0.3, 2000.0 * 4.0 / 3.0 * np.pi * 0.027, velocity=tuple(30.0 * d)))
        pos64.append(p)
    b, s = ph.pack_bodies(items)
    o = ph.avbd_options(gravity=(0, -9.81, 0), dt=1.0 / 120.0, iterations=15)
    return Scene(f"wall{cols}x{rows}", b, s, containers=[ground(1000.0, x0=offset)], options=o, steps=600,
                 positions_f64=np.array(pos64, np.float64))


# ----------------------------------------------------------- test scenes
def constraints_demo():
    """demos/constraints/src/main.rs:65-149: four static anchors, five kicked
    cubes, one joint of each kind; gravity -3.5, 16 iterations."""
    P = [(-7.0, 1.6, 0.0), (-7.0, 0.0, 0.0), (-2.5, 1.6, 0.0), (-1.7, 0.2, 0.0), (-2.2, -1.0, 0.0),
         (2.2, 1.7, 0.0), (2.2, 2.05, 0.0), (6.5, 1.7, 0.0), (6.5, -0.2, 0.0)]
    kick = {1: ((9.2, 4.4, 5.0), (0.0, 0.8, 0.0)), 3: ((-5.4, 4.0, 5.0), (0.0, 0.7, 0.0)),
            4: ((5.7, 4.2, 4.0), (0.0, -0.5, 0.0)), 6: ((5.0, 4.0, 4.8), (0.0, 0.0, 1.2)),
            8: ((-5.8, 5.5, 4.0), (0.0, 0.6, 0.0))}
    items = []
    for i, p in enumerate(P):
        if i in kick:
            items.append(ph.cube(p, 0.3, 1.0, velocity=kick[i][0], angular_velocity=kick[i][1]))
        else:
            items.append(ph.cube(p, 0.4, 0.0))
    b, s = ph.pack_bodies(items)
    js = ph.pack_joints([ph.spring(0, 1, (0, 0, 0), (0, 0, 0), 12.0, 1.6), ph.rod(2, 3, (0, 0, 0), (0, 0, 0), 1.6),
                         ph.rod(3, 4, (0, 0, 0), (0, 0, 0), 1.4),
                         ph.ball_socket(5, 6, (0, 0, 0), (0.0, -0.3, 0.0)),
                         ph.rope(7, 8, (0, 0, 0), (0, 0, 0), 1.5)])
    o = ph.avbd_options(gravity=(0, -3.5, 0), iterations=16)
    return Scene("constraints_demo", b, s, constraints=js, options=o, steps=60)


def box_demo(count=48, seed=6):
    """demos/avbd_box/src/main.rs:85-172 style: cubes, tetrahedra and spheres
    with random velocities inside a 2 m container (alpha 0.8)."""
    rng = np.random.default_rng(0x5EED + seed)
    corners = np.array([(0.0, -0.707, -1.0), (0.866025, -0.707, 0.5), (-0.866025, -0.707, 0.5),
                        (0.0, 0.707, 0.0)], np.float32) * np.float32(0.55)
    items, placed = [], []
    for i in range(count):
        for _ in range(256):
            c = rng.uniform(-1.6, 1.6, 3)
            if all(np.sum((c - p) ** 2) > 0.75 ** 2 for p in placed):
                break
        placed.append(c)
        vel = rng.uniform(-0.9, 0.9, 3)
        ang = rng.uniform(-1.2, 1.2, 3)
        if i < count // 8:
            items.append(ph.cube(c, 0.4, 1.0, velocity=vel, angular_velocity=ang))
        elif i < count // 4:
            items.append(ph.tetrahedron(c, corners, 1.0, velocity=vel, angular_velocity=ang))
        else:
            items.append(ph.sphere(c, 0.3, 1.0, velocity=vel, angular_velocity=ang))
    b, s = ph.pack_bodies(items)
    o = ph.avbd_options(alpha=0.8)
    return Scene("box_demo", b, s, containers=[ph.container((0, 0, 0), 2.0)], options=o, steps=60)


def pack(scenes):
    """Pack independent scenes into one world (per-scene body offsets)."""
    items_b, items_s, joints, offsets, conts, hulls = [], [], [], [0], [], []
    hbase = 0
    for sc in scenes:
        base = offsets[-1]
        b = sc.bodies.copy()
        if sc.hull_vertices is not None and len(sc.hull_vertices):
            mask = b["shape"]["tag"] == abi.HULL
            b["shape"]["pad"][mask, 0] += hbase
            hulls.append(sc.hull_vertices)
            hbase += len(sc.hull_vertices)
        items_b.append(b)
        items_s.append(sc.state)
        j = sc.constraints.copy()
        j["a"] += base
        j["b"] += base
        joints.append(j)
        offsets.append(base + sc.n)
        # no container: an infinite box never produces wall rows
        conts.append(sc.containers[0] if sc.containers else ph.container((0, 0, 0), float("inf")))
    return Scene("packed", np.concatenate(items_b), np.concatenate(items_s), constraints=np.concatenate(joints),
                 scene_offsets=np.array(offsets, np.uint32), containers=conts,
                 hull_vertices=np.concatenate(hulls) if hulls else None, options=scenes[0].options,
                 steps=scenes[0].steps)
