"""FP64 and split-precision worlds on the GPU.

Each precision mode is checked against the oracle instantiated with the same
precision (<double, double> for FP64, <double, float> for the split mode),
bit for bit, and the split mode's purpose is checked on a wall far from the
origin: FP64 poses and inertial targets with FP32 Hessians must track the
all-FP64 run far more closely than the all-FP32 run does."""
import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, compute, scenes

pytestmark = pytest.mark.gpu


def _world(sc, **cfg):
    hv = sc.hull_vertices
    cap = compute.capacity(sc.n, max_pairs=max(64, 40 * sc.n), max_contacts=max(256, 200 * sc.n),
                           max_joints=max(1, len(sc.constraints)), max_scenes=sc.n_scenes,
                           max_hull_vertices=max(1, len(hv) if hv is not None else 1))
    w = compute.World(cap, **cfg)
    w.upload(sc.bodies, sc.state, **sc.upload_kwargs())
    return w


@pytest.mark.parametrize("precision", [abi.PREC_SPLIT, abi.PREC_F64])
def test_precision_world_matches_same_precision_oracle(precision):
    # the 1080-body field is above the FP64 shared-memory tree size (1024)
    for sc in [scenes.pyramid(levels=4), scenes.box_demo(), scenes.constraints_demo(),
               scenes.mixed_pile(n=400, extent=5.0), scenes.cube_field(nx=12, nz=10, ny=9)]:
        ow = O.World(sc, precision=precision)
        ow.step(sc.options, 20)
        rp, rq = ow.download_f64()
        with _world(sc, precision=precision) as w:
            w.step(sc.options, 20)
            gp, gq = w.download_f64()
            st = w.stats()
        assert st["error_flags"] == 0
        assert np.array_equal(gp, rp), (sc.name, precision, np.abs(gp - rp).max())
        assert np.array_equal(gq, rq), (sc.name, precision)


def _errors(offset, steps, n_bricks):
    sc = scenes.wall_throw(cols=12, rows=8, projectiles=6, offset=offset)
    res = {}
    for prec in (abi.PREC_F32, abi.PREC_SPLIT, abi.PREC_F64):
        with _world(sc, precision=prec) as w:
            w.step(sc.options, steps)
            res[prec] = w.download_f64()[0]
    e32 = np.abs(res[abi.PREC_F32] - res[abi.PREC_F64]).max(axis=1)
    esp = np.abs(res[abi.PREC_SPLIT] - res[abi.PREC_F64]).max(axis=1)
    return e32, esp


def test_split_precision_tracks_fp64_far_from_the_origin():
    """At x = 1e5 m an FP32 pose is quantised to ~8 mm.  In flight (no
    contacts) the split mode stays at the FP64 trajectory while FP32 drifts
    by centimetres; in the contact-rich wall the split error at x = 1e5 is
    the same as at the origin (the remaining difference is the FP32 Hessian
    in a chaotic stack, not the coordinates)."""
    nb = 12 * 8
    e32, esp = _errors(1.0e5, 30, nb)
    assert esp[nb:].max() < 1e-5, esp[nb:].max()          # projectiles in flight
    assert e32[nb:].max() > 1e-3, e32[nb:].max()
    _, esp0 = _errors(0.0, 30, nb)
    assert esp[:nb].max() < 2.0 * esp0[:nb].max() + 1e-6, (esp[:nb].max(), esp0[:nb].max())
    assert esp.max() < 0.2 * e32.max(), (esp.max(), e32.max())
