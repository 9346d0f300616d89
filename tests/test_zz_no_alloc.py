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


def _noalloc_call(torch, L, state, pos, quat, rows, cons, off, idx, ro, alias_state=False):
    """One call on caller-owned device copies; returns (status, outputs)."""
    n, m = len(state), len(rows)
    d_state, d_pos, d_quat = _dev(torch, state), _dev(torch, pos), _dev(torch, quat)
    d_rows, d_cons, d_off, d_idx = _dev(torch, rows), _dev(torch, cons), _dev(torch, off), _dev(torch, idx)
    d_opos = torch.empty(n * 12, dtype=torch.uint8, device="cuda")
    d_oquat = torch.empty(n * 16, dtype=torch.uint8, device="cuda")
    d_ostate = d_state if alias_state else torch.empty(n * abi.BODY_STATE.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.dio_avbd_solve_noalloc(d_state.data_ptr(), d_pos.data_ptr(), d_quat.data_ptr(), n,
                                  d_rows.data_ptr() if m else None, m, d_cons.data_ptr() if len(cons) else None,
                                  len(cons), d_off.data_ptr(), d_idx.data_ptr() if len(idx) else None,
                                  ctypes.byref(ro), d_opos.data_ptr(), d_oquat.data_ptr(), d_ostate.data_ptr(),
                                  stream)
    return rc, (_host(d_opos, n * 12, np.float32).reshape(n, 3), _host(d_oquat, n * 16, np.float32).reshape(n, 4),
                _host(d_ostate, n * abi.BODY_STATE.itemsize, abi.BODY_STATE),
                _host(d_rows, m * abi.CONTACT.itemsize, abi.CONTACT))


def _noalloc_step(torch, L, *args, **kw):
    rc, out = _noalloc_call(torch, L, *args, **kw)
    assert rc == abi.DIO_OK, L.dio_status_string(rc)
    return out


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


def _check_against_context(got, ref, rows_present):
    got_pos, got_quat, got_state, got_rows = got
    assert np.array_equal(got_pos, ref["positions"])
    assert np.array_equal(got_quat, ref["orientations"])
    assert np.array_equal(got_state["vel"][:, :3], ref["velocities"])
    assert np.array_equal(got_state["ang"][:, :3], ref["angular_velocities"])
    assert np.array_equal(got_state["prev_vel"][:, :3], ref["prev_velocities"])
    if rows_present:
        assert np.array_equal(got_rows["lambda"][:, :3], ref["lambda"])
        assert np.array_equal(got_rows["penalty"][:, :3], ref["penalty"])


def test_noalloc_output_state_may_alias_the_input_state():
    torch = pytest.importorskip("torch")
    L = abi.lib()
    sc = scenes.box_demo(count=40)
    rows, off, idx = _inputs(sc)
    ro = ph.run_options(sc.options)
    args = (sc.state.copy(), sc.bodies["position"][:, :3].copy(), sc.bodies["orientation"].copy(), rows.copy(),
            sc.constraints, off, idx, ro)
    ref = _ctx_step(*args)
    got = _noalloc_step(torch, L, *args, alias_state=True)
    _check_against_context(got, ref, True)


def test_noalloc_rejects_out_of_range_indices():
    """A contact body, a CSR range or a joint body beyond the caller's arrays
    is DIO_ERR_INVALID, found before any kernel dereferences it."""
    torch = pytest.importorskip("torch")
    L = abi.lib()
    sc = scenes.constraints_demo()
    rows, off, idx = _inputs(sc)
    ro = ph.run_options(sc.options)
    n, m = sc.n, len(rows)
    assert m > 0 and len(sc.constraints) > 0
    base = (sc.state, sc.bodies["position"][:, :3].copy(), sc.bodies["orientation"].copy())
    bad_rows = rows.copy()
    bad_rows["a"][0] = n + 5
    rc, _ = _noalloc_call(torch, L, *base, bad_rows, sc.constraints, off, idx, ro)
    assert rc == abi.DIO_ERR_INVALID
    bad_off = off.copy()
    bad_off[-1] = 2 * m + 1
    rc, _ = _noalloc_call(torch, L, *base, rows.copy(), sc.constraints, bad_off, idx, ro)
    assert rc == abi.DIO_ERR_INVALID
    bad_cons = sc.constraints.copy()
    bad_cons["b"][0] = n
    rc, _ = _noalloc_call(torch, L, *base, rows.copy(), bad_cons, off, idx, ro)
    assert rc == abi.DIO_ERR_INVALID
    # and the next valid call is unaffected
    ref = _ctx_step(*base, rows.copy(), sc.constraints, off, idx, ro)
    got = _noalloc_step(torch, L, *base, rows.copy(), sc.constraints, off, idx, ro)
    _check_against_context(got, ref, True)


def test_noalloc_reports_a_non_finite_state():
    """A NaN velocity turns the solved pose non-finite: DIO_ERR_NONFINITE, as
    the context-based solve reports it."""
    torch = pytest.importorskip("torch")
    L = abi.lib()
    sc = scenes.box_demo(count=8)
    rows, off, idx = _inputs(sc)
    ro = ph.run_options(sc.options)
    st = sc.state.copy()
    dyn = np.flatnonzero(st["inv_mass"] != 0)
    st["vel"][dyn[0], 0] = np.nan
    rc, _ = _noalloc_call(torch, L, st, sc.bodies["position"][:, :3].copy(), sc.bodies["orientation"].copy(),
                          rows.copy(), sc.constraints, off, idx, ro)
    assert rc == abi.DIO_ERR_NONFINITE
    with compute.AvbdCompute(sc.n, max(64, len(rows)), max_joints=1) as ac:
        with pytest.raises(abi.DioError):
            ac.run(st, sc.bodies["position"][:, :3].copy(), sc.bodies["orientation"].copy(), rows.copy(),
                   sc.constraints, off, idx, ro)


_RESET_CHILD = r"""
import ctypes, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from diomedes_gb300 import abi
L = abi.lib()
rt = None
for name in ("libcudart.so.13", "libcudart.so.12", "libcudart.so"):
    try:
        rt = ctypes.CDLL(name)
        break
    except OSError:
        pass
assert rt is not None
rt.cudaMalloc.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_size_t]
rt.cudaMemcpy.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int]
rt.cudaFree.argtypes = [ctypes.c_void_p]
data = np.load(sys.argv[2])
ro = abi.RunOptions.from_buffer_copy(data["ro"].tobytes())
arrays = [data[k] for k in ("state", "pos", "quat", "rows", "cons", "off", "idx")]
n, m, nj = len(data["state"]), len(data["rows"]), len(data["cons"])

def dev(a):
    raw = np.ascontiguousarray(a).view(np.uint8).reshape(-1)
    p = ctypes.c_void_p()
    assert rt.cudaMalloc(ctypes.byref(p), max(1, raw.size)) == 0
    if raw.size:
        assert rt.cudaMemcpy(p, raw.ctypes.data, raw.size, 1) == 0
    return p

def host(p, nbytes):
    out = np.empty(nbytes, np.uint8)
    assert rt.cudaMemcpy(out.ctypes.data, p, nbytes, 2) == 0
    return out

results = []
for call in range(2):
    d = [dev(a) for a in arrays]
    opos, oquat, ost = dev(np.zeros(n * 12, np.uint8)), dev(np.zeros(n * 16, np.uint8)), dev(arrays[0])
    rc = L.dio_avbd_solve_noalloc(d[0], d[1], d[2], n, d[3], m, d[4] if nj else None, nj, d[5], d[6],
                                  ctypes.byref(ro), opos, oquat, ost, None)
    assert rc == 0, rc
    results.append(np.concatenate([host(opos, n * 12), host(oquat, n * 16),
                                   host(ost, n * abi.BODY_STATE.itemsize), host(d[3], m * abi.CONTACT.itemsize)]))
    # a new context on the same device: the scratch address must be looked up again
    assert rt.cudaDeviceReset() == 0
np.save(sys.argv[3], np.stack(results))
"""


def test_noalloc_after_a_device_reset_in_a_fresh_process(tmp_path):
    """The scratch address is cached per CUDA context: a call made after
    cudaDeviceReset (a new context on the same device) looks it up again and
    returns the same results.  Runs in a child process that owns its device
    memory through cudaMalloc (this process's allocator would not survive the
    reset)."""
    import os
    import subprocess
    import sys

    pytest.importorskip("torch")
    sc = scenes.box_demo(count=40)
    rows, off, idx = _inputs(sc)
    ro = ph.run_options(sc.options)
    state, pos, quat = sc.state.copy(), sc.bodies["position"][:, :3].copy(), sc.bodies["orientation"].copy()
    inp = tmp_path / "in.npz"
    np.savez(inp, state=state, pos=pos, quat=quat, rows=rows, cons=sc.constraints, off=off, idx=idx,
             ro=np.frombuffer(bytes(ro), np.uint8))
    out = tmp_path / "out.npy"
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    p = subprocess.run([sys.executable, "-c", _RESET_CHILD, root, str(inp), str(out)], capture_output=True,
                       text=True, timeout=300)
    assert p.returncode == 0, p.stdout + p.stderr
    res = np.load(out)
    assert np.array_equal(res[0], res[1])
    ref = _ctx_step(state, pos, quat, rows, sc.constraints, off, idx, ro)
    n = sc.n
    got_pos = res[0][: n * 12].view(np.float32).reshape(n, 3)
    got_quat = res[0][n * 12: n * 28].view(np.float32).reshape(n, 4)
    assert np.array_equal(got_pos, ref["positions"])
    assert np.array_equal(got_quat, ref["orientations"])
