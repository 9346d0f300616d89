"""Failure detection on the GPU without faulting it: a bounded device wait
that runs out, and malformed uploads rejected on the host before any kernel
reads them.  Every case leaves the context usable, which the tests check by
stepping on and comparing with the oracle."""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, compute, scenes

pytestmark = pytest.mark.gpu


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def _world(sc, **cfg):
    cap = compute.capacity(sc.n, max_pairs=max(64, 40 * sc.n), max_contacts=max(256, 200 * sc.n),
                           max_joints=max(1, len(sc.constraints)), max_scenes=sc.n_scenes,
                           max_hull_vertices=max(1, len(sc.hull_vertices) if sc.hull_vertices is not None else 1))
    w = compute.World(cap, **cfg)
    w.upload(sc.bodies, sc.state, **sc.upload_kwargs())
    return w


def test_epa_wait_running_out_reports_timeout_and_the_world_steps_on():
    """The EPA waits (bounded) for the bulk copies that stage hull vertices in
    shared memory.  With its first wait given no polls the wait runs out at
    once: the step reports DIO_ERR_TIMEOUT, while the second wait (full
    budget) still lets the copies land, so the pair is still solved from the
    staged vertices.  The state equals the oracle's after the timed-out step
    and after a normal step with the default budget restored."""
    sc = scenes.mixed_pile(n=600, extent=6.0)  # 334 hull pairs in contact at step 1
    ow = O.World(sc)
    with _world(sc) as w:
        w.configure(debug_flags=abi.DEBUG_EPA_NO_FIRST_WAIT)
        with pytest.raises(abi.DioError) as e:
            w.step(sc.options, 1)
        assert e.value.status == abi.DIO_ERR_TIMEOUT
        ow.step(sc.options, 1)
        gb, gs = w.download()
        rb, rs = ow.download()
        assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))
        w.configure(debug_flags=0)
        w.step(sc.options, 1)
        ow.step(sc.options, 1)
        gb, gs = w.download()
        rb, rs = ow.download()
        assert w.stats()["error_flags"] == 0
        assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))


def test_world_upload_rejects_hull_ranges_beyond_the_pool():
    """A hull body whose vertex range runs past the hull-vertex pool is
    DIO_ERR_INVALID before anything is copied; the world uploaded before it
    is untouched and steps as the oracle does."""
    sc = scenes.mixed_pile(n=60, extent=3.0)
    nh = len(sc.hull_vertices)
    bad = sc.bodies.copy()
    i = int(np.flatnonzero(bad["shape"]["tag"] == abi.HULL)[0])
    bad["shape"]["pad"][i, 0] = nh - 1  # first + count > nh
    with _world(sc) as w:
        hv = np.ascontiguousarray(sc.hull_vertices, np.float32)
        d = abi.WorldDesc()
        d.n_bodies = sc.n
        d.n_hull_vertices = nh
        d.bodies = bad.ctypes.data
        d.state = sc.state.ctypes.data
        d.hull_vertices = hv.ctypes.data
        assert w.L.dio_world_upload(w.h, ctypes.byref(d)) == abi.DIO_ERR_INVALID
        bad["shape"]["pad"][i, 0] = 0xFFFFFFFF  # a 32-bit wrap of first + count is caught too
        assert w.L.dio_world_upload(w.h, ctypes.byref(d)) == abi.DIO_ERR_INVALID
        w.step(sc.options, 2)
        gb, gs = w.download()
    ow = O.World(sc)
    ow.step(sc.options, 2)
    rb, rs = ow.download()
    assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))
