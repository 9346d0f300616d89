"""CUDA world step vs the oracle at the configurations the measurements use.

Bit for bit through the C ABI (the library and the oracle evaluate the same
expressions in the same order without contraction):
  * the 10-level, 55-cube pyramid, 1 and 60 steps, with the reference's
    4-contact manifold and the 8-contact extension (which yields more than
    four rows per pair once the stack settles);
  * the 32 x 32 x 8 cube field, 1 and 60 steps with 8 contacts per pair (the
    jittered, randomly oriented cubes give face clips of more than 4
    points), and one step with 4;
  * the bench's own 1024-scene batch, one full step, and its first 128
    scenes for 60 steps, in both solve launches (one scene-chunk launch,
    and init / primal / dual / recover launched per phase);
  * one step of the 50,000-body mixed convex pile and of the 200,000-brick
    wall at x = 1e5 m (FP32, and the FP32/FP64 split against the split
    oracle).
The oracle runs on every host core (the same Jacobi semantics, identical
results for any thread count)."""
import os

import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, compute, scenes

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def _capacity(sc, pairs_per_body=8, rows_per_body=16):
    return compute.capacity(sc.n, max_pairs=max(1024, pairs_per_body * sc.n),
                            max_contacts=max(4096, rows_per_body * sc.n),
                            max_joints=max(1, len(sc.constraints)), max_scenes=sc.n_scenes,
                            max_hull_vertices=max(1, len(sc.hull_vertices) if sc.hull_vertices is not None else 1))


def _compare(sc, steps_list, precision=0, contacts_per_pair=4, batched_solver=abi.SOLVE_AUTO, cap=None):
    ow = O.World(sc, precision=precision, contacts_per_pair=contacts_per_pair, threads=THREADS)
    with compute.World(cap or _capacity(sc), precision=precision) as w:
        w.configure(contacts_per_pair=contacts_per_pair, batched_solver=batched_solver)
        w.upload(sc.bodies, sc.state, **sc.upload_kwargs())
        done = 0
        for steps in steps_list:
            w.step(sc.options, steps - done)
            ow.step(sc.options, steps - done)
            done = steps
            gb, gs = w.download()
            rb, rs = ow.download()
            gc, rc = w.contacts(), ow.contacts()
            assert w.stats()["error_flags"] == 0
            assert len(gc) == len(rc), (sc.name, steps)
            assert np.array_equal(_bits(gb), _bits(rb)), (sc.name, steps)
            assert np.array_equal(_bits(gs), _bits(rs)), (sc.name, steps)
            assert np.array_equal(_bits(gc), _bits(rc)), (sc.name, steps)
            if precision:
                gp, gq = w.download_f64()
                rp, rq = ow.download_f64()
                assert np.array_equal(gp, rp) and np.array_equal(gq, rq), (sc.name, steps)
    return rc


def _max_rows_per_pair(rows):
    pr = rows[rows["b"] != 0xFFFFFFFF]
    if not len(pr):
        return 0
    _, cnt = np.unique(pr["a"].astype(np.int64) << 32 | pr["b"].astype(np.int64), return_counts=True)
    return int(cnt.max())


@pytest.mark.parametrize("contacts_per_pair", [4, 8])
def test_pyramid_55_cubes(contacts_per_pair):
    sc = scenes.pyramid(levels=10)
    assert sc.n == 55
    rows = _compare(sc, [1, 60], contacts_per_pair=contacts_per_pair)
    if contacts_per_pair == 8:
        assert _max_rows_per_pair(rows) > 4
    else:
        assert _max_rows_per_pair(rows) <= 4


def test_cube_field_32x32x8():
    sc = scenes.cube_field(nx=32, nz=32, ny=8)
    assert sc.n == 8192
    cap = _capacity(sc, 24, 24)  # 16 pairs and 12 rows per body by step 60
    rows = _compare(sc, [1, 60], contacts_per_pair=8, cap=cap)
    assert _max_rows_per_pair(rows) > 4
    _compare(sc, [1], cap=cap)


@pytest.fixture(scope="module")
def bench_batch():
    return scenes.batched(n_scenes=1024)


@pytest.mark.parametrize("batched_solver", [abi.SOLVE_AUTO, abi.SOLVE_PER_PHASE])
def test_bench_batch_one_full_step(bench_batch, batched_solver):
    sc = bench_batch
    assert sc.n_scenes == 1024 and sc.n > 400_000
    _compare(sc, [1], batched_solver=batched_solver, cap=_capacity(sc, 2, 4))


@pytest.mark.parametrize("batched_solver", [abi.SOLVE_AUTO, abi.SOLVE_PER_PHASE])
def test_bench_batch_first_128_scenes_60_steps(bench_batch, batched_solver):
    sc = bench_batch.select(range(128))
    _compare(sc, [1, 60], batched_solver=batched_solver, cap=_capacity(sc, 2, 4))


def test_mixed_pile_50k_one_step():
    sc = scenes.mixed_pile(n=50000)
    _compare(sc, [1], cap=_capacity(sc, 4, 8))


@pytest.mark.parametrize("precision", [abi.PREC_F32, abi.PREC_SPLIT])
def test_wall_throw_200k_one_step(precision):
    sc = scenes.wall_throw(cols=400, rows=500, projectiles=1000)
    assert sc.n == 201_000
    _compare(sc, [1], precision=precision, cap=_capacity(sc, 3, 8))
