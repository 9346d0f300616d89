"""Host-side mirror of the reference's physics API (engine/src/physics/*.rs).

Bodies, shapes, joints and options are built as numpy records in the exact
byte layouts of the C ABI, with the reference's own constructors and
defaults (f32 arithmetic as in the Rust code):
  AvbdBody::{sphere, cube, tetrahedron}  engine/src/physics/gpu.rs:32-94
  AvbdOptions::default                   engine/src/physics/gpu.rs:140-155
  Spring / Rod / BallSocket / Rope       engine/src/physics/constraints.rs:10-124
  GpuShape::{sphere, cube, tetrahedron}  engine/src/render/compute.rs:41-72
  constraints_from_avbd                  engine/src/render/gpu_physics.rs:149-193
"""
import numpy as np

from . import abi

f32 = np.float32

DEFAULT_ROD_STIFFNESS = f32(1000.0)
DEFAULT_SOCKET_STIFFNESS = f32(1000.0)
DEFAULT_ROPE_STIFFNESS = f32(1000.0)


# ----------------------------------------------------------------- shapes
def shape_sphere(radius):
    s = np.zeros((), abi.SHAPE)
    s["tag"] = abi.SPHERE
    s["corners"][0, 0] = radius
    return s


def shape_cube(half_extent):
    s = np.zeros((), abi.SHAPE)
    s["tag"] = abi.CUBE
    s["corners"][0, :3] = half_extent
    return s


def shape_tetrahedron(corners):
    s = np.zeros((), abi.SHAPE)
    s["tag"] = abi.TETRAHEDRON
    s["corners"][:, :3] = np.asarray(corners, np.float32)
    return s


def shape_box(half_extents):
    """Per-axis box (extension; the reference's cube SAT uses one half extent)."""
    s = np.zeros((), abi.SHAPE)
    s["tag"] = abi.BOX
    s["corners"][0, :3] = np.asarray(half_extents, np.float32)
    return s


def shape_hull(first_vertex, vertex_count):
    """Convex vertex hull (extension): vertices live in the world's hull pool."""
    s = np.zeros((), abi.SHAPE)
    s["tag"] = abi.HULL
    s["pad"][0] = first_vertex
    s["pad"][1] = vertex_count
    return s


# ----------------------------------------------------------------- bodies
def _inv(mass):
    mass = f32(mass)
    return f32(1.0) / mass if mass > 0 else f32(0.0)


def body(position, shape, mass, inv_moment, orientation=(0, 0, 0, 1), velocity=(0, 0, 0),
         angular_velocity=(0, 0, 0), friction=0.8):
    """One body as a (GpuBody, GpuAvbdBodyState) record pair."""
    b = np.zeros((), abi.BODY)
    b["position"][:3] = position
    b["orientation"][:] = orientation
    b["shape"] = shape
    s = np.zeros((), abi.BODY_STATE)
    s["vel"][:3] = velocity
    s["ang"][:3] = angular_velocity
    s["inv_moment"][:3] = inv_moment
    s["inv_mass"] = _inv(mass)
    s["friction"] = friction
    return b, s


def sphere(position, radius, mass, **kw):
    """AvbdBody::sphere, engine/src/physics/gpu.rs:32-50."""
    m, r = f32(mass), f32(radius)
    im = f32(1.0) / (f32(0.4) * m * r * r) if m > 0 else f32(0.0)
    return body(position, shape_sphere(r), m, (im, im, im), **kw)


def cube(position, half_extent, mass, **kw):
    """AvbdBody::cube, engine/src/physics/gpu.rs:52-70."""
    m, h = f32(mass), f32(half_extent)
    im = f32(1.0) / ((f32(2.0) / f32(3.0)) * m * h * h) if m > 0 else f32(0.0)
    return body(position, shape_cube(h), m, (im, im, im), **kw)


def tetrahedron(position, corners, mass, **kw):
    """AvbdBody::tetrahedron, engine/src/physics/gpu.rs:72-94 (sphere inertia
    of the farthest corner)."""
    m = f32(mass)
    c = np.asarray(corners, np.float32)
    r = f32(0.0)
    for k in range(4):
        r = max(r, f32(np.sqrt(f32(c[k, 0] * c[k, 0] + c[k, 1] * c[k, 1]) + c[k, 2] * c[k, 2])))
    im = f32(1.0) / (f32(0.4) * m * r * r) if m > 0 else f32(0.0)
    return body(position, shape_tetrahedron(c), m, (im, im, im), **kw)


def box(position, half_extents, mass, **kw):
    """Per-axis box (extension): solid-box inertia m (h_j^2 + h_k^2) / 3."""
    m = f32(mass)
    h = np.asarray(half_extents, np.float32)
    if m > 0:
        im = tuple(f32(3.0) / (m * (h[j] * h[j] + h[k] * h[k])) for j, k in ((1, 2), (0, 2), (0, 1)))
    else:
        im = (0.0, 0.0, 0.0)
    return body(position, shape_box(h), m, im, **kw)


def hull(position, first_vertex, vertices, mass, **kw):
    """Convex hull (extension) with the tetrahedron's sphere-of-farthest-
    vertex inertia."""
    m = f32(mass)
    v = np.asarray(vertices, np.float32)
    r = f32(np.sqrt((v[:, :3].astype(np.float64) ** 2).sum(1).max()))
    im = f32(1.0) / (f32(0.4) * m * r * r) if m > 0 else f32(0.0)
    return body(position, shape_hull(first_vertex, len(v)), m, (im, im, im), **kw)


def pack_bodies(pairs):
    bodies = np.zeros(len(pairs), abi.BODY)
    state = np.zeros(len(pairs), abi.BODY_STATE)
    for i, (b, s) in enumerate(pairs):
        bodies[i] = b
        state[i] = s
    return bodies, state


# ---------------------------------------------------------------- options
def avbd_options(**over):
    """AvbdOptions::default, engine/src/physics/gpu.rs:140-155."""
    o = abi.AvbdOptions()
    o.dt = 1.0 / 60.0
    o.gravity[:] = (0.0, -10.0, 0.0)
    o.iterations = 10
    o.alpha = 0.99
    o.beta_lin = 10000.0
    o.margin = 0.01
    o.penalty_min = 1.0
    o.penalty_max = 1e10
    o.gamma = 0.999
    o.friction = 0.8
    for k, v in over.items():
        if k == "gravity":
            o.gravity[:] = v
        else:
            setattr(o, k, v)
    return o


def run_options(o):
    """The AvbdRunOptions subset of AvbdOptions (demos/*/main.rs build it)."""
    r = abi.RunOptions()
    r.dt = o.dt
    r.gravity[:] = tuple(o.gravity)
    r.alpha = o.alpha
    r.beta_lin = o.beta_lin
    r.penalty_max = o.penalty_max
    r.iterations = o.iterations
    return r


def container(center, half_extent, rotation=(0, 0, 0, 1)):
    c = abi.Container()
    c.center[:] = center
    c.half_extent = half_extent
    c.rotation[:] = rotation
    return c


# ----------------------------------------------------------------- joints
def _joint(a, b, kind, anchor_a, anchor_b, aw, bw):
    j = np.zeros((), abi.CONSTRAINT)
    j["a"], j["b"], j["kind"] = a, b, kind
    j["anchor_a"][:3] = anchor_a
    j["anchor_a"][3] = aw
    j["anchor_b"][:3] = anchor_b
    j["anchor_b"][3] = bw
    return j


def spring(a, b, anchor_a, anchor_b, stiffness, rest_length):
    """Spring::new (constraints.rs:19-37) serialised as in constraints_from_avbd."""
    return _joint(a, b, abi.SPRING, anchor_a, anchor_b, rest_length, stiffness)


def rod(a, b, anchor_a, anchor_b, rest_length, stiffness=DEFAULT_ROD_STIFFNESS):
    return _joint(a, b, abi.ROD, anchor_a, anchor_b, rest_length, stiffness)


def ball_socket(a, b, anchor_a, anchor_b, stiffness=DEFAULT_SOCKET_STIFFNESS):
    return _joint(a, b, abi.BALL_SOCKET, anchor_a, anchor_b, 0.0, stiffness)


def rope(a, b, anchor_a, anchor_b, max_length, stiffness=DEFAULT_ROPE_STIFFNESS):
    return _joint(a, b, abi.ROPE, anchor_a, anchor_b, max_length, stiffness)


JOINT_NAMES = {abi.SPRING: "spring", abi.ROD: "rod", abi.BALL_SOCKET: "ball and socket", abi.ROPE: "rope"}


def joint_name(j):
    """Constraint::name, constraints.rs:142-149."""
    return JOINT_NAMES[int(j["kind"])]


def quat_rotate(q, v):
    """q v q* (float32), as the kernels compute it."""
    q = np.asarray(q, np.float32)
    v = np.asarray(v, np.float32)
    b = q[:3]
    t = np.cross(b, v).astype(np.float32) * f32(2.0)
    return (v + t * q[3] + np.cross(b, t)).astype(np.float32)


def endpoints(j, bodies):
    """Constraint::endpoints, constraints.rs:127-140."""
    a, b = int(j["a"]), int(j["b"])
    if a >= len(bodies) or b >= len(bodies):
        return None
    pa = bodies[a]["position"][:3] + quat_rotate(bodies[a]["orientation"], j["anchor_a"][:3])
    pb = bodies[b]["position"][:3] + quat_rotate(bodies[b]["orientation"], j["anchor_b"][:3])
    return pa.astype(np.float32), pb.astype(np.float32)


def pack_joints(js):
    out = np.zeros(len(js), abi.CONSTRAINT)
    for i, j in enumerate(js):
        out[i] = j
    return out
