"""Writes reference_cases.json: the known answers of the reference's own unit
tests on this path, as data.

The reference is Rust (and rust-gpu shaders) and cannot be built or imported
here, so its tests are read as text: every case below carries the file:line
range it comes from and the literal fragments of that source (inputs and
assertions) it transcribes.  Give the reference checkout's root as the
argument, or in DIO_REFERENCE_ROOT, to check that each range still contains
its fragments before the fixture is written; without the checkout the
fixture is written from the transcription alone.

    python tests/golden/make_reference_cases.py [REFERENCE_ROOT]
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = [
    # ---- SAT manifold, engine/gpu_physics/narrowphase/src/cuboid.rs
    {"id": "cube_helper", "kind": "none", "source": "engine/gpu_physics/narrowphase/src/cuboid.rs:385-400",
     "anchors": ["tag: CUBE", "Vec4::new(0.5, 0.5, 0.5, 0.0)", "Quat::IDENTITY"],
     "input": {"half_extent": 0.5}, "expect": {}},
    {"id": "touching_cubes_have_zero_penetration", "kind": "sat",
     "source": "engine/gpu_physics/narrowphase/src/cuboid.rs:403-408",
     "anchors": ["collide_manifold(&cube(Vec3::ZERO), &cube(Vec3::X))", "manifold.depth.abs() < 1.0e-6",
                 "manifold.normal.dot(Vec3::X) > 0.99"],
     "input": {"a": [0.0, 0.0, 0.0], "b": [1.0, 0.0, 0.0]},
     "expect": {"contact": True, "depth": 0.0, "depth_tol": 1e-6, "normal_dot_x_min": 0.99}},
    {"id": "overlapping_cubes_report_four_face_contacts", "kind": "sat",
     "source": "engine/gpu_physics/narrowphase/src/cuboid.rs:410-417",
     "anchors": ["Vec3::new(0.9, 0.0, 0.0)", "(manifold.depth - 0.1).abs() < 1.0e-6",
                 "manifold.normal.dot(Vec3::X) > 0.99", "assert_eq!(manifold.count, 4)"],
     "input": {"a": [0.0, 0.0, 0.0], "b": [0.9, 0.0, 0.0]},
     "expect": {"contact": True, "depth": 0.1, "depth_tol": 1e-6, "normal_dot_x_min": 0.99, "count": 4}},
    {"id": "separated_cubes_have_no_contact", "kind": "sat",
     "source": "engine/gpu_physics/narrowphase/src/cuboid.rs:419-422",
     "anchors": ["Vec3::new(1.1, 0.0, 0.0)", "is_none()"],
     "input": {"a": [0.0, 0.0, 0.0], "b": [1.1, 0.0, 0.0]}, "expect": {"contact": False}},
    # ---- support, engine/src/physics/shape.rs
    {"id": "sphere_support_tracks_direction", "kind": "support", "source": "engine/src/physics/shape.rs:53-64",
     "anchors": ["Shape::Sphere(2.0)", "Vec3::new(1.0, 0.0, 0.0)", "Vec3::new(2.0, 0.0, 0.0)",
                 "Vec3::new(0.0, -3.0, 0.0)", "Vec3::new(0.0, -2.0, 0.0)"],
     "input": {"shape": "sphere", "radius": 2.0, "dirs": [[1, 0, 0], [0, -3, 0]]},
     "expect": {"points": [[2, 0, 0], [0, -2, 0]]}},
    {"id": "cube_support_is_a_corner", "kind": "support", "source": "engine/src/physics/shape.rs:66-74",
     "anchors": ["Shape::Cube(0.5)", "Vec3::new(1.0, 1.0, 1.0)", "Vec3::splat(0.5)", "Vec3::new(-1.0, 1.0, 0.0)",
                 "Vec3::new(-0.5, 0.5, 0.5)"],
     "input": {"shape": "cube", "half_extent": 0.5, "dirs": [[1, 1, 1], [-1, 1, 0]]},
     "expect": {"points": [[0.5, 0.5, 0.5], [-0.5, 0.5, 0.5]]}},
    {"id": "tetrahedron_support_is_the_farthest_corner", "kind": "support_tetra",
     "source": "engine/src/physics/shape.rs:76-94",
     "anchors": ["Vec3::new(1.0, 1.0, 1.0)", "Vec3::new(1.0, -1.0, -1.0)", "Vec3::new(-1.0, 1.0, -1.0)",
                 "Vec3::new(-1.0, -1.0, 1.0)", "assert_eq!(point.x, 1.0);", "Vec3::new(-1.0, -1.0, 0.0)"],
     "input": {"corners": [[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], "tie_dir": [1, 0, 0],
               "dirs": [[-1, -1, 0]]},
     "expect": {"tie_x": 1.0, "points": [[-1, -1, 1]]}},
    # ---- container floor, engine/src/physics/gpu.rs
    {"id": "penetrating_cube_gets_four_floor_contacts", "kind": "container",
     "source": "engine/src/physics/gpu.rs:420-433",
     "anchors": ["center: Vec3::new(0.0, 4.0, 0.0)", "half_extent: 4.0", "Vec3::new(0.0, 0.49, 0.0), 0.5, 1.0",
                 "assert_eq!(contacts.len(), 4);", "contact.normal == Vec3::Y", "contact.r_a.y < -0.49"],
     "input": {"center": [0.0, 4.0, 0.0], "half_extent": 4.0, "cube_at": [0.0, 0.49, 0.0], "h": 0.5,
               "mass": 1.0},
     "expect": {"count": 4, "normal": [0.0, 1.0, 0.0], "r_a_y_max": -0.49}},
    # ---- joints, engine/src/physics/constraints.rs and engine/src/render/gpu_physics.rs
    {"id": "endpoints_apply_body_rotation_and_local_anchors", "kind": "endpoints",
     "source": "engine/src/physics/constraints.rs:158-174",
     "anchors": ["AvbdBody::cube(Vec3::ZERO, 0.5, 0.0)", "AvbdBody::cube(Vec3::new(2.0, 0.0, 0.0), 0.5, 1.0)",
                 "Quat::from_rotation_z(90.0f32.to_radians())", "Vec3::new(0.5, 0.0, 0.0)",
                 "Vec3::new(0.0, -0.5, 0.0)", "assert_eq!(b, Vec3::new(2.5, -0.0, 0.0));"],
     "input": {"a_pos": [0, 0, 0], "b_pos": [2, 0, 0], "b_rot_z_deg": 90.0, "anchor_a": [0.5, 0, 0],
               "anchor_b": [0, -0.5, 0]},
     # exact in the reference (glam's quaternion product); the restatement's
     # product order leaves ~3e-8 in y, so the fixture carries a tolerance
     "expect": {"a": [0.5, 0.0, 0.0], "b": [2.5, 0.0, 0.0], "tol": 1e-6}},
    {"id": "constraint_names_cover_all_kinds", "kind": "names", "source": "engine/src/physics/constraints.rs:176-186",
     "anchors": ['["spring", "rod", "ball and socket", "rope"]'],
     "input": {}, "expect": {"names": ["spring", "rod", "ball and socket", "rope"]}},
    {"id": "constraint_records_keep_shader_layout_and_kinds", "kind": "records",
     "source": "engine/src/render/gpu_physics.rs:701-721",
     "anchors": ["Spring::new(0, 1, Vec3::ZERO, Vec3::ZERO, 2.0, 1.0)", "Rope::new(0, 1, Vec3::ZERO, Vec3::ZERO, 3.0)",
                 "size_of::<[f32; 12]>()", "assert_eq!(records[3].anchor_a.w, 3.0);"],
     "input": {"spring": [2.0, 1.0], "rod": 1.0, "rope": 3.0},
     "expect": {"record_bytes": 48, "kinds": ["spring", "rod", "ball_socket", "rope"], "rope_anchor_a_w": 3.0}},
]


def lines_of(root, source):
    path, rng = source.rsplit(":", 1)
    lo, hi = (int(x) for x in rng.split("-"))
    with open(os.path.join(root, path)) as f:
        return "".join(f.readlines()[lo - 1:hi])


def check(root):
    bad = []
    for c in CASES:
        text = lines_of(root, c["source"])
        bad += [(c["id"], a) for a in c["anchors"] if a not in text]
    return bad


def main():
    # the reference checkout: the first argument or DIO_REFERENCE_ROOT; with
    # neither, the fixture is written without checking the cited fragments
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DIO_REFERENCE_ROOT", "")
    checked = bool(root) and os.path.isdir(root)
    if checked:
        bad = check(root)
        if bad:
            for cid, a in bad:
                print(f"{cid}: fragment not found in the cited lines: {a}")
            sys.exit(1)
    out = {"checked_against_reference_sources": checked, "cases": CASES}
    with open(os.path.join(HERE, "reference_cases.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")
    print(f"{len(CASES)} cases written" + (" (fragments found in the cited sources)" if checked else ""))


if __name__ == "__main__":
    main()
