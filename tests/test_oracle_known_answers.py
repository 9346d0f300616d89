"""The reference's own unit tests, ported, run against the CPU oracle, plus
analytic cases that pin the restated arithmetic where the reference has no
test (free fall, sphere overlap, resting force balance, warm start)."""
import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, physics as ph, scenes


def cube_at(x, y=0.0, z=0.0, h=0.5, mass=1.0, q=(0, 0, 0, 1)):
    return ph.cube((x, y, z), h, mass, orientation=q)


def pair01():
    return np.array([(0, 1)], abi.PAIR)


# ---- engine/gpu_physics/narrowphase/src/cuboid.rs:403-422
def test_touching_cubes_have_zero_penetration():
    b, _ = ph.pack_bodies([cube_at(0.0), cube_at(1.0)])
    s = O.narrow(b, pair01())
    v = s[s["valid"] != 0]
    assert len(v) >= 1
    assert abs(v["depth"][0]) < 1e-6
    assert v["normal"][0, 0] > 0.99


def test_overlapping_cubes_report_four_face_contacts():
    b, _ = ph.pack_bodies([cube_at(0.0), cube_at(0.9)])
    s = O.narrow(b, pair01())
    v = s[s["valid"] != 0]
    assert abs(v["depth"][0] - 0.1) < 1e-6
    assert v["normal"][0, 0] > 0.99
    assert len(v) == 4


def test_separated_cubes_have_no_contact():
    b, _ = ph.pack_bodies([cube_at(0.0), cube_at(1.1)])
    assert (O.narrow(b, pair01())["valid"] == 0).all()


# ---- engine/src/physics/shape.rs:53-95 (GPU rule: first maximal corner)
def test_sphere_support_tracks_direction():
    s = ph.shape_sphere(2.0)
    assert np.array_equal(O.support(s, (1, 0, 0)), [2, 0, 0])
    assert np.array_equal(O.support(s, (0, -3, 0)), [0, -2, 0])


def test_cube_support_is_a_corner():
    s = ph.shape_cube(0.5)
    assert np.array_equal(O.support(s, (1, 1, 1)), [0.5, 0.5, 0.5])
    assert np.array_equal(O.support(s, (-1, 1, 0)), [-0.5, 0.5, 0.5])


def test_tetrahedron_support_is_the_farthest_corner():
    c = [(1, 1, 1), (1, -1, -1), (-1, 1, -1), (-1, -1, 1)]
    s = ph.shape_tetrahedron(c)
    p = O.support(s, (1, 0, 0))
    assert p[0] == 1.0
    # corners 0 and 1 tie along +x; the GPU keeps the first (support.rs:232-236)
    assert np.array_equal(p, [1, 1, 1])
    assert np.array_equal(O.support(s, (-1, -1, 0)), [-1, -1, 1])


# ---- engine/src/physics/gpu.rs:420-433
def test_penetrating_cube_gets_four_floor_contacts():
    container = ph.container((0.0, 4.0, 0.0), 4.0)
    b, s = ph.pack_bodies([cube_at(0.0, y=0.49, mass=1.0)])
    rows, off, idx = O.prepare_contacts(b, s, np.zeros(0, abi.CONTACT_OUT), None, container, ph.avbd_options())
    assert len(rows) == 4
    assert np.array_equal(rows["normal"][:, :3], np.tile([0, 1, 0], (4, 1)).astype(np.float32))
    assert (rows["r_a"][:, 1] < -0.49).all()
    assert rows["b"].tolist() == [abi.CONTAINER] * 4
    assert off.tolist() == [0, 4] and idx.tolist() == [0, 1, 2, 3]


# ---- engine/src/physics/constraints.rs:158-186
def test_endpoints_apply_body_rotation_and_local_anchors():
    q = (0.0, 0.0, np.sin(np.pi / 4), np.cos(np.pi / 4))
    b, _ = ph.pack_bodies([cube_at(0.0, mass=0.0), cube_at(2.0, q=q)])
    j = ph.ball_socket(0, 1, (0.5, 0, 0), (0, -0.5, 0))
    pa, pb = ph.endpoints(j, b)
    assert np.allclose(pa, [0.5, 0, 0], atol=1e-6)
    assert np.allclose(pb, [2.5, 0, 0], atol=1e-6)


def test_constraint_names_cover_all_kinds():
    js = [ph.spring(0, 1, (0, 0, 0), (0, 0, 0), 1.0, 1.0), ph.rod(0, 1, (0, 0, 0), (0, 0, 0), 1.0),
          ph.ball_socket(0, 1, (0, 0, 0), (0, 0, 0)), ph.rope(0, 1, (0, 0, 0), (0, 0, 0), 1.0)]
    assert [ph.joint_name(j) for j in js] == ["spring", "rod", "ball and socket", "rope"]


# ---- engine/src/render/gpu_physics.rs:701-721
def test_constraint_records_keep_shader_layout_and_kinds():
    js = ph.pack_joints([ph.spring(0, 1, (0, 0, 0), (0, 0, 0), 2.0, 1.0), ph.rod(0, 1, (0, 0, 0), (0, 0, 0), 1.0),
                         ph.ball_socket(0, 1, (0, 0, 0), (0, 0, 0)), ph.rope(0, 1, (0, 0, 0), (0, 0, 0), 3.0)])
    assert abi.CONSTRAINT.itemsize == 48
    assert js["kind"].tolist() == [abi.SPRING, abi.ROD, abi.BALL_SOCKET, abi.ROPE]
    assert js["anchor_a"][3, 3] == 3.0


# ---- analytic cases (no reference test covers them)
def test_free_fall_matches_closed_form():
    """No contacts: the primal solution is the inertial target x + v dt + g dt^2."""
    b, s = ph.pack_bodies([ph.sphere((0, 10, 0), 0.5, 2.0, velocity=(1, 0, 0))])
    ro = ph.run_options(ph.avbd_options(gravity=(0, -9.81, 0)))
    out = O.avbd_run(s, b["position"][:, :3], b["orientation"], np.zeros(0, abi.CONTACT),
                     np.zeros(0, abi.CONSTRAINT), np.zeros(2, np.uint32), np.zeros(0, np.uint32), ro)
    dt = 1.0 / 60.0
    assert np.allclose(out["positions"][0], [dt, 10 - 9.81 * dt * dt, 0], atol=1e-5)
    assert np.allclose(out["velocities"][0], [1, -9.81 * dt, 0], atol=1e-3)


def test_sphere_pair_analytic_contact():
    b, _ = ph.pack_bodies([ph.sphere((0, 0, 0), 0.5, 1.0), ph.sphere((0.8, 0, 0), 0.5, 1.0)])
    v = O.narrow(b, pair01())
    assert v["valid"][0] == 1 and (v["valid"][1:] == 0).all()
    assert abs(v["depth"][0] - 0.2) < 1e-6
    assert np.allclose(v["normal"][0, :3], [1, 0, 0])
    assert np.allclose(v["point_a"][0, :3], [0.5, 0, 0]) and np.allclose(v["point_b"][0, :3], [0.3, 0, 0])


def test_gjk_epa_tetrahedron_vs_sphere_depth():
    corners = scenes.regular_tetrahedron(0.4)
    b, _ = ph.pack_bodies([ph.tetrahedron((0, 0, 0), corners, 1.0), ph.sphere((0, -0.35, 0), 0.3, 1.0)])
    v = O.narrow(b, pair01())
    assert v["valid"][0] == 1
    # the sphere overlaps the face opposite... depth is positive and small
    assert 0.0 < v["depth"][0] < 0.3


def test_resting_cube_force_balance():
    """A cube resting on the floor: after steps the floor rows carry the
    weight, sum(lambda_n) -> -m g dt^2 scale (force in the penalty units)."""
    # the pyramid workload's stiff parameters: alpha 0.95, beta 1e5, k0 1e4
    # (with alpha 0.99 only 1% of the penetration is corrected per step)
    sc = scenes.Scene("rest", *ph.pack_bodies([cube_at(0.0, y=0.5, mass=2.0)]), containers=[scenes.ground()],
                      options=ph.avbd_options(gravity=(0, -10, 0), alpha=0.95, beta_lin=1e5, penalty_min=1e4))
    w = O.World(sc)
    w.step(sc.options, 120)
    rows = w.contacts()
    assert len(rows) == 4
    total = float(rows["lambda"][:, 0].sum())
    # lambda is the contact force: the four floor rows carry -m g
    assert total == pytest.approx(-2.0 * 10.0, rel=1e-3)
    bb, _ = w.download()
    # rests on the floor within the 0.01 m margin
    assert abs(bb["position"][0, 1] - 0.5) < 0.015


def test_warm_start_hands_last_previous_row_to_first_new_row():
    """finalize_contacts: HashMap insert keeps the LAST previous row of a key,
    remove hands it to the FIRST new row with that key only."""
    b, s = ph.pack_bodies([cube_at(0.0), cube_at(0.9)])
    slots = O.narrow(b, pair01())
    prev = np.zeros(3, abi.CONTACT)
    prev["a"], prev["b"] = 0, 1
    prev["lambda"][:, 0] = [-1.0, -2.0, -3.0]
    prev["penalty"][:, :3] = [[10, 10, 10], [20, 20, 20], [30, 30, 30]]
    o = ph.avbd_options()
    rows, _, _ = O.prepare_contacts(b, s, slots, prev, None, o)
    ag = np.float32(o.alpha) * np.float32(o.gamma)
    assert rows["lambda"][0, 0] == np.float32(-3.0) * ag
    assert rows["penalty"][0, 0] == np.float32(30.0) * np.float32(o.gamma)
    assert (rows["lambda"][1:, 0] == 0).all()
    assert (rows["penalty"][1:, 0] == np.float32(o.penalty_min)).all()


def test_dense_and_sort_and_sweep_pair_sets_agree():
    sc = scenes.cube_field(nx=6, nz=6, ny=3)
    d, nd = O.broad(sc.bodies, sap=False)
    s, ns = O.broad(sc.bodies, sap=True)
    assert nd == ns and nd > 0
    assert np.array_equal(d, s)
