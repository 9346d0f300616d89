"""The reference's own unit tests, ported, run against the CPU oracle, plus
analytic cases that pin the restated arithmetic where the reference has no
test (free fall, sphere overlap, resting force balance, warm start)."""
import json
import math
import os

import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, physics as ph, scenes


def cube_at(x, y=0.0, z=0.0, h=0.5, mass=1.0, q=(0, 0, 0, 1)):
    return ph.cube((x, y, z), h, mass, orientation=q)


def pair01():
    return np.array([(0, 1)], abi.PAIR)


# ---- the reference's own unit tests on this path, as data (tests/golden/
# reference_cases.json, written by tests/golden/make_reference_cases.py from
# the cited reference sources)
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_cases.json")
with open(GOLDEN) as _f:
    CASES = [c for c in json.load(_f)["cases"] if c["kind"] != "none"]


def _run_case(c):
    i, e = c["input"], c["expect"]
    k = c["kind"]
    if k == "sat":
        b, _ = ph.pack_bodies([cube_at(*i["a"]), cube_at(*i["b"])])
        v = O.narrow(b, pair01())
        v = v[v["valid"] != 0]
        if not e["contact"]:
            assert len(v) == 0
            return
        assert len(v) >= 1
        assert abs(v["depth"][0] - e["depth"]) < e["depth_tol"]
        assert v["normal"][0, 0] > e["normal_dot_x_min"]
        if "count" in e:
            assert len(v) == e["count"]
    elif k == "support":
        s = ph.shape_sphere(i["radius"]) if i["shape"] == "sphere" else ph.shape_cube(i["half_extent"])
        for d, p in zip(i["dirs"], e["points"]):
            assert np.array_equal(O.support(s, d), p)
    elif k == "support_tetra":
        s = ph.shape_tetrahedron(i["corners"])
        p = O.support(s, i["tie_dir"])
        assert p[0] == e["tie_x"] and float(np.dot(p, i["tie_dir"])) == e["tie_x"]
        # corners 0 and 1 tie along +x; the GPU rule keeps the first (support.rs:232-236)
        assert np.array_equal(p, i["corners"][0])
        for d, q in zip(i["dirs"], e["points"]):
            assert np.array_equal(O.support(s, d), q)
    elif k == "container":
        container = ph.container(tuple(i["center"]), i["half_extent"])
        b, st = ph.pack_bodies([cube_at(*i["cube_at"], h=i["h"], mass=i["mass"])])
        rows, off, idx = O.prepare_contacts(b, st, np.zeros(0, abi.CONTACT_OUT), None, container,
                                            ph.avbd_options())
        assert len(rows) == e["count"]
        assert np.array_equal(rows["normal"][:, :3], np.tile(e["normal"], (e["count"], 1)).astype(np.float32))
        assert (rows["r_a"][:, 1] < e["r_a_y_max"]).all()
        assert rows["b"].tolist() == [abi.CONTAINER] * e["count"]
        assert off.tolist() == [0, e["count"]] and idx.tolist() == list(range(e["count"]))
    elif k == "endpoints":
        half = np.radians(i["b_rot_z_deg"]) / 2
        q = (0.0, 0.0, np.sin(half), np.cos(half))
        b, _ = ph.pack_bodies([cube_at(*i["a_pos"], mass=0.0), cube_at(*i["b_pos"], q=q)])
        j = ph.ball_socket(0, 1, tuple(i["anchor_a"]), tuple(i["anchor_b"]))
        pa, pb = ph.endpoints(j, b)
        assert np.allclose(pa, e["a"], atol=e["tol"]) and np.allclose(pb, e["b"], atol=e["tol"])
    elif k == "names":
        js = [ph.spring(0, 1, (0, 0, 0), (0, 0, 0), 1.0, 1.0), ph.rod(0, 1, (0, 0, 0), (0, 0, 0), 1.0),
              ph.ball_socket(0, 1, (0, 0, 0), (0, 0, 0)), ph.rope(0, 1, (0, 0, 0), (0, 0, 0), 1.0)]
        assert [ph.joint_name(j) for j in js] == e["names"]
    elif k == "records":
        js = ph.pack_joints([ph.spring(0, 1, (0, 0, 0), (0, 0, 0), *i["spring"]),
                             ph.rod(0, 1, (0, 0, 0), (0, 0, 0), i["rod"]),
                             ph.ball_socket(0, 1, (0, 0, 0), (0, 0, 0)),
                             ph.rope(0, 1, (0, 0, 0), (0, 0, 0), i["rope"])])
        assert abi.CONSTRAINT.itemsize == e["record_bytes"]
        kinds = {"spring": abi.SPRING, "rod": abi.ROD, "ball_socket": abi.BALL_SOCKET, "rope": abi.ROPE}
        assert js["kind"].tolist() == [kinds[x] for x in e["kinds"]]
        assert js["anchor_a"][3, 3] == e["rope_anchor_a_w"]
    else:
        raise AssertionError(f"unknown case kind {k}")


@pytest.mark.parametrize("case", CASES, ids=[c["id"] for c in CASES])
def test_reference_known_answer(case):
    _run_case(case)


def test_golden_fixture_names_its_sources():
    with open(GOLDEN) as f:
        data = json.load(f)
    assert data["checked_against_reference_sources"]
    for c in data["cases"]:
        path, rng = c["source"].rsplit(":", 1)
        assert path.endswith(".rs") and "-" in rng and c["anchors"], c["id"]


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


def test_spring_hangs_at_its_analytic_extension():
    """A Hookean spring (k 1e3, rest 0.5) holding 1 kg from a static body
    settles at rest + m g / k below it (the primal's implicit steps damp the
    oscillation)."""
    k, rest, m, g = 1000.0, 0.5, 1.0, 10.0
    b, s = ph.pack_bodies([ph.sphere((0, 10, 0), 0.2, 0.0), ph.sphere((0, 10 - rest, 0), 0.2, m)])
    cons = ph.pack_joints([ph.spring(0, 1, (0, 0, 0), (0, 0, 0), k, rest)])
    sc = scenes.Scene("spring", b, s, constraints=cons, options=ph.avbd_options(gravity=(0, -g, 0)))
    w = O.World(sc)
    w.step(sc.options, 600)
    bb, _ = w.download()
    assert bb["position"][1, 1] == pytest.approx(10 - rest - m * g / k, abs=1e-4)


def _box_on_slope(theta_deg, mu, steps, **opt):
    """A unit cube resting on a container floor tilted by theta about z (the
    box aligned with the floor); its centre before and after each run of steps."""
    th = math.radians(theta_deg)
    half, h = 50.0, 0.5
    q = (0.0, 0.0, math.sin(th / 2), math.cos(th / 2))
    up = np.array([-math.sin(th), math.cos(th), 0.0])
    p0 = -(half - h) * up
    b, s = ph.pack_bodies([ph.cube(tuple(p0), h, 1.0, orientation=q)])
    sc = scenes.Scene("slope", b, s, containers=[ph.container((0, 0, 0), half, q)],
                      options=ph.avbd_options(gravity=(0, -9.81, 0), friction=mu, **opt))
    w = O.World(sc)
    out = []
    for k in steps:
        w.step(sc.options, k)
        out.append(w.download()[0]["position"][0, :3].astype(np.float64))
    return p0, out


def test_box_slides_down_a_steep_slope_at_the_coulomb_rate():
    """40 degrees, mu 0.5 (tan 40 > mu): after 2 s the box has slid
    g (sin - mu cos) t^2 / 2 (5.10 m), within 3 %."""
    p0, (p,) = _box_on_slope(40.0, 0.5, [120])
    th = math.radians(40.0)
    expect = 0.5 * 9.81 * (math.sin(th) - 0.5 * math.cos(th)) * 2.0 ** 2
    assert float(np.linalg.norm(p - p0)) == pytest.approx(expect, rel=0.03)


def test_box_sticks_on_a_shallow_slope():
    """10 degrees, mu 0.5 (tan 10 < mu), the stiff parameters of the pyramid
    workload: after settling the box does not move (under 1 mm in 2 s)."""
    p0, (a, b) = _box_on_slope(10.0, 0.5, [60, 120], alpha=0.95, beta_lin=1e5, penalty_min=1e4)
    assert float(np.linalg.norm(b - a)) < 1e-3


def test_rope_is_free_while_slack_and_holds_at_its_length():
    """A rope (max length 1.0, k 1e3) from a static body: while slack the body
    follows the free-fall recurrence of the implicit step (v -= g dt, y += v
    dt); once taut it hangs at the length plus m g / k."""
    g, dt = 10.0, 1.0 / 60.0
    b, s = ph.pack_bodies([ph.sphere((0, 10, 0), 0.1, 0.0), ph.sphere((0, 9.5, 0), 0.1, 1.0)])
    cons = ph.pack_joints([ph.rope(0, 1, (0, 0, 0), (0, 0, 0), 1.0)])
    sc = scenes.Scene("rope", b, s, constraints=cons, options=ph.avbd_options(gravity=(0, -g, 0)))
    w = O.World(sc)
    v, y = 0.0, 9.5
    for _ in range(6):
        w.step(sc.options, 1)
        v -= g * dt
        y += v * dt
        assert w.download()[0]["position"][1, 1] == pytest.approx(y, abs=1e-5)
    w.step(sc.options, 600)
    assert w.download()[0]["position"][1, 1] == pytest.approx(10.0 - 1.0 - 1.0 * g / float(ph.DEFAULT_ROPE_STIFFNESS),
                                                             abs=1e-4)


def test_pendulum_keeps_its_length_and_gains_no_energy():
    """A body on a ball socket 0.8 m from a static pivot, released level with
    it: every sampled position stays 0.8 m (plus the joint's stretch under
    load, k 1e3) from the pivot and never rises above the release height."""
    b, s = ph.pack_bodies([ph.sphere((0, 10, 0), 0.1, 0.0), ph.sphere((0.8, 10, 0), 0.1, 1.0)])
    cons = ph.pack_joints([ph.ball_socket(0, 1, (0, 0, 0), (-0.8, 0, 0))])
    sc = scenes.Scene("pendulum", b, s, constraints=cons, options=ph.avbd_options(gravity=(0, -10.0, 0)))
    w = O.World(sc)
    for _ in range(20):
        w.step(sc.options, 60)
        p = w.download()[0]["position"][1, :3].astype(np.float64)
        r = float(np.linalg.norm(p - np.array([0.0, 10.0, 0.0])))
        assert 0.79 < r < 0.84
        assert p[1] <= 10.0 + 1e-4


def test_gjk_epa_box_sphere_face_contact():
    """A unit cube and a sphere (r 0.3) overlapping through a face: GJK + EPA
    give the face normal (a -> b), depth h + r - d, and witnesses on the cube's
    face and on the sphere's surface (EPA tolerance 1e-4)."""
    for centre, axis in (((0, 0.7, 0), 1), ((0.7, 0, 0), 0), ((0, 0, -0.75), 2)):
        b, _ = ph.pack_bodies([ph.cube((0, 0, 0), 0.5, 1.0), ph.sphere(centre, 0.3, 1.0)])
        v = O.narrow(b, pair01())
        d = abs(centre[axis])
        sign = np.sign(centre[axis])
        n = np.zeros(3)
        n[axis] = sign
        assert v["valid"][0] == 1
        assert v["depth"][0] == pytest.approx(0.5 + 0.3 - d, abs=1e-4)
        assert np.allclose(v["normal"][0, :3], n, atol=1e-4)
        assert np.allclose(v["point_a"][0, :3], 0.5 * n, atol=1e-4)
        assert np.allclose(v["point_b"][0, :3], (d - 0.3) * n, atol=1e-4)
