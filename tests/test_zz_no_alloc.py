"""dio_avbd_solve_noalloc against dio_avbd_submit / dio_avbd_read.

The no-allocation entry point serves callers that cannot call cudaMalloc
while they step the solver (a host whose device memory comes from another
allocator, or a real-time loop that must not allocate once running).  The
test owns all device memory (through torch, as such a caller would through
its own allocator), calls the entry point twice in a row -- the second call
continuing from the first call's outputs -- and checks both results against
the context-based solve, which must agree exactly (the tolerance used by
the other AVBD parity tests: bit for bit).  This file is collected last so a
run that stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, compute, physics as ph, scenes

pytestmark = pytest.mark.gpu


def _inputs(sc):
    pairs, _ = O.broad(sc.bodies)
    slots = O.narrow(sc.bodies, pairs)
    cont = sc.containers[0] if sc.containers else None
    rows, off, idx = O.prepare_contacts(sc.bodies, sc.state, slots, None, cont, sc.options)
    return rows, off, idx


def _dev(torch, arr):
    """Copy a numpy record array into caller-owned device memory (bytes)."""
    raw = np.ascontiguousarray(arr).view(np.uint8).reshape(-1)
    t = torch.empty(max(1, raw.size), dtype=torch.uint8, device="cuda")
    if raw.size:
        t[: raw.size].copy_(torch.from_numpy(raw.copy()))
    return t


def _host(t, nbytes, dtype):
    return t[:nbytes].cpu().numpy().view(dtype).copy()


def _noalloc_step(torch, L, state, pos, quat, rows, cons, off, idx, ro):
    n, m = len(state), len(rows)
    d_state, d_pos, d_quat = _dev(torch, state), _dev(torch, pos), _dev(torch, quat)
    d_rows, d_cons, d_off, d_idx = _dev(torch, rows), _dev(torch, cons), _dev(torch, off), _dev(torch, idx)
    d_opos = torch.empty(n * 12, dtype=torch.uint8, device="cuda")
    d_oquat = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    d_ostate = torch.empty(n * abi.BODY_STATE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.dio_avbd_solve_noalloc(d_state.data_ptr(), d_pos.data_ptr(), d_quat.data_ptr(), n,
                                  d_rows.data_ptr() if m else None, m, d_cons.data_ptr() if len(cons) else None,
                                  len(cons), d_off.data_ptr(), d_idx.data_ptr() if len(idx) else None,
                                  ctypes.byref(ro), d_opos.data_ptr(), d_oquat.data_ptr(), d_ostate.data_ptr(),
                                  stream)
    assert rc == abi.DIO_OK, L.dio_status_string(rc)
    return (_host(d_opos, n * 12, np.float32).reshape(n, 3), _host(d_oquat, n * 16, np.float32).reshape(n, 4),
            _host(d_ostate, n * abi.BODY_STATE.itemsize, abi.BODY_STATE),
            _host(d_rows, m * abi.CONTACT.itemsize, abi.CONTACT))


def _ctx_step(state, pos, quat, rows, cons, off, idx, ro):
    with compute.AvbdCompute(len(state), max(64, len(rows)), max_joints=max(1, len(cons))) as ac:
        return ac.run(state, pos, quat, rows, cons, off, idx, ro)


@pytest.mark.parametrize("make", [lambda: scenes.pyramid(levels=4), scenes.constraints_demo,
                                  lambda: scenes.box_demo(count=40)])
def test_noalloc_matches_context_solve_on_two_calls(make):
    torch = pytest.importorskip("torch")
    L = abi.lib()
    sc = make()
    rows, off, idx = _inputs(sc)
    ro = ph.run_options(sc.options)
    state, pos, quat = sc.state.copy(), sc.bodies["position"][:, :3].copy(), sc.bodies["orientation"].copy()
    cur_rows = rows.copy()
    for call in range(2):
        ref = _ctx_step(state, pos, quat, cur_rows, sc.constraints, off, idx, ro)
        got_pos, got_quat, got_state, got_rows = _noalloc_step(torch, L, state, pos, quat, cur_rows,
                                                               sc.constraints, off, idx, ro)
        assert np.array_equal(got_pos, ref["positions"]), call
        assert np.array_equal(got_quat, ref["orientations"]), call
        assert np.array_equal(got_state["vel"][:, :3], ref["velocities"]), call
        assert np.array_equal(got_state["ang"][:, :3], ref["angular_velocities"]), call
        assert np.array_equal(got_state["prev_vel"][:, :3], ref["prev_velocities"]), call
        if len(cur_rows):
            assert np.array_equal(got_rows["lambda"][:, :3], ref["lambda"]), call
            assert np.array_equal(got_rows["penalty"][:, :3], ref["penalty"]), call
        # continue from this call's outputs (the scratch keeps the last call's contents)
        state, pos, quat, cur_rows = got_state, got_pos, got_quat, got_rows


def test_noalloc_rejects_sizes_beyond_its_scratch():
    pytest.importorskip("torch")
    L = abi.lib()
    ro = ph.run_options(ph.avbd_options())
    rc = L.dio_avbd_solve_noalloc(None, None, None, 4097, None, 0, None, 0, None, None, ctypes.byref(ro), None,
                                  None, None, None)
    assert rc == abi.DIO_ERR_CAPACITY
    rc = L.dio_avbd_solve_noalloc(None, None, None, 8, None, 16385, None, 0, None, None, ctypes.byref(ro), None,
                                  None, None, None)
    assert rc == abi.DIO_ERR_CAPACITY
