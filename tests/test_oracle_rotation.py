"""How far the rounding of the rotation alone moves a step.

The reference rotates every lever arm, anchor, support direction and box
axis with glam's Quat * Vec3 (glam 0.33.3 mul_vec3: with b = q.xyz,
v (w w - b.b) + 2 (v.b) b + 2 w (b x v)), and the oracle and the kernels
evaluate that form term for term.  An algebraically equal form (v + w t +
b x t with t = 2 b x v) rounds differently; so may glam's SIMD paths on
other hosts.  From one identical state after 30 steps, one step with either
form must agree within the spec's one-step tolerance of 1e-5 relative
(positions and quaternion components relative to max(|value|, 1), lambdas
relative to the step's largest |lambda|), while 60 steps from the start
show how quickly contact stacks amplify a one-ulp difference (chaotic
divergence; the reason longer horizons are compared per body within stated
tolerances, not bit for bit)."""
import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import scenes

ONE_STEP_REL = 1e-5


def _rel(a, b, floor):
    return float((np.abs(a - b) / np.maximum(np.abs(b), floor)).max())


def _state_after(sc, steps):
    w = O.World(sc)
    w.step(sc.options, steps)
    b, s = w.download()
    return scenes.Scene(f"{sc.name}@{steps}", b, s, constraints=sc.constraints, scene_offsets=sc.scene_offsets,
                        containers=sc.containers, options=sc.options)


@pytest.mark.parametrize("make", [lambda: scenes.pyramid(levels=10), scenes.constraints_demo,
                                  lambda: scenes.box_demo(count=40), lambda: scenes.cube_field(nx=8, nz=8, ny=4),
                                  lambda: scenes.batched(n_scenes=16)])
def test_one_step_with_either_rotation_rounding_agrees_within_tolerance(make):
    sc = _state_after(make(), 30)
    glam, alt = O.World(sc), O.World(sc, variant="rotate_tq")
    glam.step(sc.options, 1)
    alt.step(sc.options, 1)
    gb, _ = glam.download()
    ab, _ = alt.download()
    gc, ac = glam.contacts(), alt.contacts()
    assert len(gc) == len(ac) and len(gc) > 0, sc.name  # same contact rows
    assert _rel(ab["position"][:, :3], gb["position"][:, :3], 1.0) <= ONE_STEP_REL
    assert _rel(ab["orientation"], gb["orientation"], 1.0) <= ONE_STEP_REL
    lam = np.abs(gc["lambda"][:, :3]).max()
    assert np.abs(gc["lambda"][:, :3] - ac["lambda"][:, :3]).max() <= ONE_STEP_REL * lam


def test_contact_stacks_amplify_the_rotation_rounding_over_60_steps():
    """Both forms agree bit for bit on the first step of the 10-level
    pyramid (no contact yet) and drift apart as the stack settles: the
    difference after 60 steps is many orders above the first step's."""
    sc = scenes.pyramid(levels=10)
    glam, alt = O.World(sc), O.World(sc, variant="rotate_tq")
    glam.step(sc.options, 1)
    alt.step(sc.options, 1)
    assert np.array_equal(glam.download()[0], alt.download()[0])
    glam.step(sc.options, 59)
    alt.step(sc.options, 59)
    d = np.abs(glam.download()[0]["position"][:, :3] - alt.download()[0]["position"][:, :3]).max()
    assert d > 1e-4
