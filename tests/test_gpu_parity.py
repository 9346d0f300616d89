"""CUDA path vs the CPU oracle through the C ABI, on identical inputs.

Integer results (pair sets, slot validity, row counts, CSR) must match bit
for bit; float results are compared bit for bit where the kernels evaluate
the same expressions in the same order (they are built with --fmad=false),
and otherwise within the stated tolerance."""
import numpy as np
import pytest

import oracle_lib as O
from diomedes_gb300 import abi, compute, physics as ph, scenes

pytestmark = pytest.mark.gpu

# one-step state tolerance (relative, with an absolute floor) for paths whose
# summation order is not forced to match the oracle's
REL_TOL = 1e-5


def small_scenes():
    return [
        scenes.pyramid(levels=4),
        scenes.constraints_demo(),
        scenes.box_demo(),
        scenes.cube_field(nx=6, nz=6, ny=3),
        scenes.mixed_pile(n=600, extent=6.0),
    ]


def _bits(a):
    return np.ascontiguousarray(a).view(np.uint8)


def test_broad_pair_sets_bit_exact():
    for sc in small_scenes():
        ref, nref = O.broad(sc.bodies, hull=sc.hull_vertices)
        with compute.NarrowPhaseCompute(sc.n, max(16, 64 * sc.n), max_hull_vertices=max(1, len(sc.hull_vertices) if sc.hull_vertices is not None else 1)) as npc:
            if sc.hull_vertices is not None:
                npc.set_hull_vertices(sc.hull_vertices)
            npc.submit_broad(sc.bodies)
            count = npc.read_pair_count()
            pairs = npc.read_pairs(count)
        assert count == nref, sc.name
        assert np.array_equal(pairs, ref), sc.name


def test_narrow_slots_bit_exact():
    for sc in small_scenes():
        pairs, _ = O.broad(sc.bodies, hull=sc.hull_vertices)
        if len(pairs) == 0:
            continue
        ref = O.narrow(sc.bodies, pairs, hull=sc.hull_vertices)
        hv = sc.hull_vertices if sc.hull_vertices is not None else np.zeros((1, 4), np.float32)
        with compute.NarrowPhaseCompute(sc.n, len(pairs), max_hull_vertices=len(hv)) as npc:
            npc.set_hull_vertices(hv)
            got = npc.run(sc.bodies, pairs)
        assert np.array_equal(got["valid"], ref["valid"]), sc.name
        assert np.array_equal(_bits(got), _bits(ref)), sc.name


def test_broad_then_narrow_on_device_pairs():
    sc = scenes.cube_field(nx=5, nz=5, ny=2)
    with compute.NarrowPhaseCompute(sc.n, 64 * sc.n) as npc:
        npc.submit_broad(sc.bodies)
        count = npc.read_pair_count()
        npc.submit_narrow(count)
        got = npc.read()
    pairs, _ = O.broad(sc.bodies)
    ref = O.narrow(sc.bodies, pairs)
    assert np.array_equal(_bits(got), _bits(ref))


def _prep_inputs(sc):
    pairs, _ = O.broad(sc.bodies, hull=sc.hull_vertices)
    slots = O.narrow(sc.bodies, pairs, hull=sc.hull_vertices)
    return slots


def test_prepare_contacts_rows_and_csr_bit_exact():
    for sc in [scenes.pyramid(levels=4), scenes.box_demo(), scenes.cube_field(nx=4, nz=4, ny=2)]:
        slots = _prep_inputs(sc)
        cont = sc.containers[0] if sc.containers else None
        o = sc.options
        rows0, off0, idx0 = O.prepare_contacts(sc.bodies, sc.state, slots, None, cont, o)
        # a previous step's rows with non-trivial lambda / penalty
        prev = rows0.copy()
        prev["lambda"][:, :3] = -np.arange(len(prev) * 3, dtype=np.float32).reshape(-1, 3)
        prev["penalty"][:, :3] = 5.0 + np.arange(len(prev) * 3, dtype=np.float32).reshape(-1, 3)
        ref, roff, ridx = O.prepare_contacts(sc.bodies, sc.state, slots, prev, cont, o)
        with compute.AvbdCompute(sc.n, max(64, 4 * len(ref) + 64), max_pairs=max(16, len(slots))) as ac:
            got, goff, gidx = ac.prepare_contacts(sc.bodies, sc.state, slots, prev, cont, o)
        assert len(got) == len(ref), sc.name
        assert np.array_equal(goff, roff) and np.array_equal(gidx, ridx), sc.name
        assert np.array_equal(_bits(got), _bits(ref)), sc.name


def _avbd_inputs(sc):
    slots = _prep_inputs(sc)
    cont = sc.containers[0] if sc.containers else None
    rows, off, idx = O.prepare_contacts(sc.bodies, sc.state, slots, None, cont, sc.options)
    return rows, off, idx


def test_avbd_run_matches_oracle():
    for sc in [scenes.pyramid(levels=4), scenes.constraints_demo(), scenes.box_demo(),
               scenes.cube_field(nx=4, nz=4, ny=2)]:
        rows, off, idx = _avbd_inputs(sc)
        ro = ph.run_options(sc.options)
        args = (sc.state, sc.bodies["position"][:, :3], sc.bodies["orientation"], rows, sc.constraints, off, idx, ro)
        ref = O.avbd_run(*args)
        with compute.AvbdCompute(sc.n, max(64, len(rows)), max_joints=max(1, len(sc.constraints))) as ac:
            got = ac.run(*args)
        for k in ref:
            assert np.array_equal(_bits(got[k]), _bits(ref[k])), (sc.name, k)


def _world(sc, **cfg):
    cap = compute.capacity(sc.n, max_pairs=max(64, 40 * sc.n), max_contacts=max(256, 200 * sc.n),
                           max_joints=max(1, len(sc.constraints)), max_scenes=sc.n_scenes,
                           max_hull_vertices=max(1, len(sc.hull_vertices) if sc.hull_vertices is not None else 1))
    w = compute.World(cap, **cfg)
    w.upload(sc.bodies, sc.state, **sc.upload_kwargs())
    return w


@pytest.mark.parametrize("steps,use_graph,batched_solver", [(1, 1, abi.SOLVE_AUTO), (60, 1, abi.SOLVE_AUTO),
                                                            (60, 0, abi.SOLVE_AUTO), (1, 1, abi.SOLVE_PER_PHASE),
                                                            (60, 1, abi.SOLVE_PER_PHASE)])
def test_world_steps_match_oracle(steps, use_graph, batched_solver):
    """SOLVE_AUTO runs each step's solve as one scene-chunk launch (every
    scene here fits a chunk), SOLVE_PER_PHASE as init / primal / dual /
    recover launches: both equal the oracle bit for bit."""
    for sc in small_scenes():
        ow = O.World(sc)
        ow.step(sc.options, steps)
        rb, rs = ow.download()
        rc = ow.contacts()
        with _world(sc, use_graph=use_graph, batched_solver=batched_solver) as w:
            for _ in range(steps):  # one dio_step per step: graph replay per call
                w.step(sc.options, 1)
            gb, gs = w.download()
            gc = w.contacts()
            st = w.stats()
        assert st["error_flags"] == 0
        assert len(gc) == len(rc), sc.name
        assert np.array_equal(_bits(gb), _bits(rb)), (sc.name, steps)
        assert np.array_equal(_bits(gs), _bits(rs)), (sc.name, steps)
        assert np.array_equal(_bits(gc), _bits(rc)), (sc.name, steps)


def _scene_with_static_overlap():
    """A pyramid plus two overlapping static boxes: their contact rows have no
    dynamic endpoint (no primal visits them; the dual still updates them)."""
    sc = scenes.pyramid(levels=4)
    extra = [ph.cube((6.0, 0.5, 0.0), 0.5, 0.0), ph.cube((6.6, 0.5, 0.0), 0.5, 0.0)]
    b, s = ph.pack_bodies(extra)
    return scenes.Scene("pyramid+static", np.concatenate([sc.bodies, b]), np.concatenate([sc.state, s]),
                        containers=sc.containers, options=sc.options)


def test_rows_without_dynamic_endpoint_match_oracle():
    """Rows between two static bodies are never visited by a primal thread
    but the dual still advances their lambda / penalty every iteration: the
    contact output matches the oracle's bits (and the rest of the world)."""
    for sc in [_scene_with_static_overlap(), scenes.box_demo()]:
        ow = O.World(sc)
        ow.step(sc.options, 12)
        with _world(sc) as w:
            w.step(sc.options, 12)
            gb, gs = w.download()
            gc = w.contacts()
        rb, rs = ow.download()
        rc = ow.contacts()
        if sc.name == "pyramid+static":
            n0 = sc.n - 2
            assert np.any((rc["a"] >= n0) & (rc["b"] >= n0)), "no static-static row"
        assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs)), sc.name
        assert np.array_equal(_bits(gc), _bits(rc)), sc.name


def test_set_state_that_changes_dynamic_bodies_rebuilds_the_list():
    """dio_world_set_state keeps the dynamic-body list unless a body turns
    static or dynamic; then the list is rebuilt and the body moves (or stops)."""
    sc = _scene_with_static_overlap()
    k = sc.n - 1  # a static box overlapping another static box
    with _world(sc) as w:
        w.step(sc.options, 2)
        b0, s0 = w.download()
        s1 = s0.copy()
        s1["inv_mass"][k] = 1.0
        s1["inv_moment"][k, :3] = 6.0
        w.set_state(None, s1)
        w.step(sc.options, 4)
        b1, s1b = w.download()
        assert not np.array_equal(b1["position"][k], b0["position"][k])  # now dynamic: it moves
        s2 = s1b.copy()
        s2["inv_mass"][k] = 0.0
        s2["inv_moment"][k, :3] = 0.0
        s2["vel"][k] = 0.0
        s2["ang"][k] = 0.0
        w.set_state(None, s2)
        w.step(sc.options, 3)
        b2, _ = w.download()
        assert np.array_equal(b2["position"][k], b1["position"][k])  # static again: it stays
        assert w.stats()["error_flags"] == 0
        # an unchanged state keeps the list: stepping matches a world stepped without it
        w.set_state(None, w.download()[1])


def _lag_scenes():
    parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo()]
    for p in parts:
        p.options = parts[0].options
    return [scenes.box_demo(), scenes.mixed_pile(n=600, extent=6.0), scenes.pack(parts)]


@pytest.mark.parametrize("use_graph", [0, 1])
def test_contact_lag_matches_oracle(use_graph):
    """contact_lag = 1 reproduces the demos' frame pipelining: the pair rows of
    step t come from the narrow phase of step t-1 (its witness points, this
    step's transforms), container rows are current.  Bit for bit against the
    oracle in the same mode, from upload and when switched on mid-run."""
    for sc in _lag_scenes():
        ow = O.World(sc, contact_lag=1)
        with _world(sc, use_graph=use_graph, contact_lag=1) as w:
            ow.step(sc.options, 1)
            w.step(sc.options, 1)
            gc, rc = w.contacts(), ow.contacts()
            assert not np.any(rc["b"] != 0xFFFFFFFF)  # no detection before the first step
            assert np.array_equal(_bits(gc), _bits(rc)), sc.name
            ow.step(sc.options, 11)
            w.step(sc.options, 11)
            gb, gs = w.download()
            gc = w.contacts()
        rb, rs = ow.download()
        assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs)), sc.name
        assert np.array_equal(_bits(gc), _bits(ow.contacts())), sc.name
        ow2 = O.World(sc)
        ow2.step(sc.options, 4)
        ow2.set_lag(1)
        ow2.step(sc.options, 6)
        with _world(sc, use_graph=use_graph) as w2:
            w2.step(sc.options, 4)
            w2.configure(contact_lag=1)
            w2.step(sc.options, 6)
            gb2, gs2 = w2.download()
        rb2, rs2 = ow2.download()
        assert np.array_equal(_bits(gb2), _bits(rb2)) and np.array_equal(_bits(gs2), _bits(rs2)), sc.name


def test_checkpoint_resume_in_contact_lag_mode():
    """A lagged world's checkpoint carries the last step's narrow slots: the
    resumed world continues bit for bit."""
    sc = _lag_scenes()[1]
    with _world(sc, contact_lag=1) as w:
        w.step(sc.options, 5)
        img = w.checkpoint()
        w.step(sc.options, 6)
        ref_b, ref_s = w.download()
    h = compute.checkpoint_header(img)
    assert h["lag_pairs"] > 0 and h["per_pair"] == 4
    cap = compute.capacity(sc.n, max_pairs=max(64, 40 * sc.n), max_contacts=max(256, 200 * sc.n),
                           max_joints=1, max_scenes=1, max_hull_vertices=len(sc.hull_vertices))
    with compute.World(cap) as w2:
        with pytest.raises(abi.DioError):  # a lagged image needs a lagged context
            w2.resume(img)
        w2.configure(contact_lag=1)
        w2.resume(img)
        w2.step(sc.options, 6)
        gb, gs = w2.download()
    assert np.array_equal(_bits(gb), _bits(ref_b)) and np.array_equal(_bits(gs), _bits(ref_s))


def test_pipelined_frames_match_synchronous_steps():
    """A frame loop of dio_step_async + dio_world_download_async into two
    alternating page-locked buffers (read frame t-1 while t computes) yields
    the same per-frame states as synchronous stepping; a device error raised
    by an asynchronous step is reported by the next synchronisation."""
    torch = pytest.importorskip("torch")
    sc = scenes.constraints_demo()
    frames = 6
    ref = []
    with _world(sc) as w:
        for _ in range(frames):
            w.step(sc.options, 1)
            ref.append(w.download())

    def pinned(dt):
        return torch.empty(sc.n * dt.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(dt)

    bufs = [(pinned(abi.BODY), pinned(abi.BODY_STATE)) for _ in range(2)]
    seen = []
    with _world(sc) as w:
        for t in range(frames):
            w.step_async(sc.options, 1)
            w.download_async(*bufs[t % 2])
            if t:
                w.synchronize()  # frame t-1's buffer is complete (and t's, here)
                seen.append((bufs[(t - 1) % 2][0].copy(), bufs[(t - 1) % 2][1].copy()))
        w.synchronize()
        seen.append((bufs[(frames - 1) % 2][0].copy(), bufs[(frames - 1) % 2][1].copy()))
        for (gb, gs), (rb, rs) in zip(seen, ref):
            assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))
        b, s = w.download()
        bad = s.copy()
        bad["vel"][1, 0] = np.nan
        w.set_state(None, bad)
        w.step_async(sc.options, 1)  # returns without waiting
        with pytest.raises(abi.DioError) as e:
            w.synchronize()
        assert e.value.status == abi.DIO_ERR_NONFINITE


def test_worlds_stepped_from_host_match_one_packed_world():
    """dio_worlds_step_host over a batch split into three worlds on three
    streams (host copies of one overlapping the others' steps) gives, frame
    by frame, the bits of the packed world stepped by set_state / dio_step /
    download; a non-finite state in one world is reported by the call."""
    torch = pytest.importorskip("torch")
    parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo(),
             scenes.cube_field(nx=3, nz=3, ny=2), scenes.mixed_pile(n=120, extent=3.0)]
    for p in parts:
        p.options = parts[0].options
    packed = scenes.pack(parts)
    frames = 5
    with _world(packed) as w:
        b, s = w.download()
        for _ in range(frames):
            w.set_state(b, s)
            w.step(packed.options, 1)
            b, s = w.download()

    def pinned(dt):
        return torch.empty(packed.n * dt.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(dt)

    hb, hs = pinned(abi.BODY), pinned(abi.BODY_STATE)
    hb[:], hs[:] = packed.bodies, packed.state
    groups, starts = packed.split(3)
    streams = [torch.cuda.Stream() for _ in groups]
    worlds = [_world(g) for g in groups]
    try:
        for wg, st in zip(worlds, streams):
            wg.set_stream(st.cuda_stream)
        vb = [hb[lo:lo + g.n] for g, lo in zip(groups, starts)]
        vs = [hs[lo:lo + g.n] for g, lo in zip(groups, starts)]
        compute.step_host(worlds, vb, vs, packed.options, 2)
        compute.step_host(worlds, vb, vs, packed.options, frames - 2)
        assert np.array_equal(_bits(hb), _bits(b)) and np.array_equal(_bits(hs), _bits(s))
        bad = hs.copy()
        bad["vel"][starts[1] + 1, 0] = np.nan
        vs[1][:] = bad[starts[1]:starts[1] + groups[1].n]
        with pytest.raises(abi.DioError) as e:
            compute.step_host(worlds, vb, vs, packed.options, 1)
        assert e.value.status == abi.DIO_ERR_NONFINITE
    finally:
        for wg in worlds:
            wg.close()


def test_transform_export_matches_the_poses():
    """Headless transform export into a device buffer: pose records are the
    downloaded poses; model matrices are translation * rotation * scale built
    from them (float32 restatement, bit for bit); a misaligned buffer is
    rejected."""
    torch = pytest.importorskip("torch")
    sc = scenes.mixed_pile(n=400, extent=5.0)
    with _world(sc) as w:
        w.step(sc.options, 5)
        b, _ = w.download()
        pose = torch.zeros((sc.n, 8), dtype=torch.float32, device="cuda")
        w.export_transforms(pose.data_ptr(), 32, abi.XFORM_POSE)
        scales = torch.linspace(0.5, 2.0, sc.n, dtype=torch.float32, device="cuda")
        mats = torch.zeros((sc.n, 20), dtype=torch.float32, device="cuda")  # 80-byte stride
        w.export_transforms(mats.data_ptr(), 80, abi.XFORM_MAT4, scales.data_ptr())
        torch.cuda.synchronize()
        with pytest.raises(abi.DioError):
            w.export_transforms(pose.data_ptr() + 4, 32, abi.XFORM_POSE)
        with pytest.raises(abi.DioError):
            w.export_transforms(pose.data_ptr(), 16, abi.XFORM_POSE)
        pose, mats, s = pose.cpu().numpy(), mats.cpu().numpy()[:, :16], scales.cpu().numpy()
    assert np.array_equal(pose[:, :3], b["position"][:, :3]) and not pose[:, 3].any()
    assert np.array_equal(pose[:, 4:], b["orientation"])
    f = np.float32
    x, y, z, w_ = (b["orientation"][:, k].astype(f) for k in range(4))
    x2, y2, z2 = x + x, y + y, z + z
    xx, xy, xz, yy, yz, zz = x * x2, x * y2, x * z2, y * y2, y * z2, z * z2
    wx, wy, wz = w_ * x2, w_ * y2, w_ * z2
    one, zero = f(1), np.zeros_like(x)
    cols = [((one - (yy + zz)) * s, (xy + wz) * s, (xz - wy) * s, zero),
            ((xy - wz) * s, (one - (xx + zz)) * s, (yz + wx) * s, zero),
            ((xz + wy) * s, (yz - wx) * s, (one - (xx + yy)) * s, zero),
            (b["position"][:, 0], b["position"][:, 1], b["position"][:, 2], np.ones_like(x))]
    want = np.stack([c for col in cols for c in col], axis=1).astype(f)
    assert np.array_equal(mats, want)


@pytest.mark.parametrize("precision", [abi.PREC_F32, abi.PREC_SPLIT, abi.PREC_F64])
def test_checkpoint_resume_continues_bit_for_bit(precision):
    """A world checkpointed after 7 steps and resumed in another context steps
    on to the same bits -- poses, state, FP64 poses and the contact rows with
    their lambda / penalty -- as the world that was never interrupted (joints,
    hulls, containers, several scenes)."""
    parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.mixed_pile(n=300, extent=5.0)]
    for p in parts:
        p.options = parts[0].options
    sc = scenes.pack(parts)
    with _world(sc, precision=precision) as w:
        w.step(sc.options, 7)
        img = w.checkpoint()
        w.step(sc.options, 9)
        ref_b, ref_s = w.download()
        ref_p, ref_q = w.download_f64()
        ref_c = w.contacts()
    h = compute.checkpoint_header(img)
    assert h["magic"] == b"DIOCKPT1" and h["version"] == 1 and h["precision"] == precision
    assert (h["n"], h["n_joints"], h["n_scenes"], h["steps"]) == (sc.n, len(sc.constraints), sc.n_scenes, 7)
    assert h["n_hull"] == len(sc.hull_vertices) and h["total_bytes"] == len(img) and h["rows"] > 0
    cap = compute.capacity(sc.n, max_pairs=max(64, 40 * sc.n), max_contacts=max(256, 200 * sc.n),
                           max_joints=max(1, len(sc.constraints)), max_scenes=sc.n_scenes,
                           max_hull_vertices=len(sc.hull_vertices))
    with compute.World(cap, precision=precision) as w2:
        w2.resume(img)
        w2.step(sc.options, 9)
        gb, gs = w2.download()
        gp, gq = w2.download_f64()
        gc = w2.contacts()
        bad = bytearray(img)
        bad[:8] = b"NOTACKPT"
        with pytest.raises(abi.DioError):
            w2.resume(bytes(bad))
        with pytest.raises(abi.DioError):
            w2.resume(img[: len(img) // 2])
    assert np.array_equal(_bits(gb), _bits(ref_b)) and np.array_equal(_bits(gs), _bits(ref_s))
    assert np.array_equal(gp, ref_p) and np.array_equal(gq, ref_q)
    assert np.array_equal(_bits(gc), _bits(ref_c))


def test_batched_world_equals_each_scene_alone():
    parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo(),
             scenes.cube_field(nx=3, nz=3, ny=2)]
    for p in parts:
        p.options = parts[0].options
    packed = scenes.pack(parts)
    with _world(packed) as w:
        w.step(packed.options, 5)
        gb, gs = w.download()
    for k, p in enumerate(parts):
        lo, hi = packed.scene_offsets[k], packed.scene_offsets[k + 1]
        if not p.containers:
            p.containers = [packed.containers[k]]
        with _world(p) as w1:
            w1.step(packed.options, 5)
            b1, s1 = w1.download()
        assert np.array_equal(_bits(gb[lo:hi]), _bits(b1)), p.name
        assert np.array_equal(_bits(gs[lo:hi]), _bits(s1)), p.name


def test_empty_inputs():
    with compute.NarrowPhaseCompute(8, 64) as npc:
        npc.submit_broad(np.zeros(0, abi.BODY))
        assert npc.read_pair_count() == 0
        assert len(npc.run(np.zeros(0, abi.BODY), np.zeros(0, abi.PAIR))) == 0
    with compute.AvbdCompute(8, 64) as ac:
        out = ac.run(np.zeros(0, abi.BODY_STATE), np.zeros((0, 3), np.float32), np.zeros((0, 4), np.float32),
                     np.zeros(0, abi.CONTACT), np.zeros(0, abi.CONSTRAINT), np.zeros(1, np.uint32),
                     np.zeros(0, np.uint32), ph.run_options(ph.avbd_options()))
        assert len(out["positions"]) == 0


def test_capacity_errors_are_reported():
    sc = scenes.cube_field(nx=4, nz=4, ny=2)
    with compute.NarrowPhaseCompute(sc.n, 4) as npc:
        npc.submit_broad(sc.bodies)
        with pytest.raises(abi.DioError) as e:
            npc.read_pair_count()
        assert e.value.status == abi.DIO_ERR_CAPACITY
    with pytest.raises(abi.DioError) as e:
        with compute.NarrowPhaseCompute(4, 64) as npc:
            npc.submit_broad(sc.bodies)
    assert e.value.status == abi.DIO_ERR_CAPACITY


def test_bad_indices_are_rejected():
    sc = scenes.pyramid(levels=2)
    with compute.NarrowPhaseCompute(sc.n, 64) as npc:
        with pytest.raises(abi.DioError) as e:
            npc.run(sc.bodies, np.array([(0, 99)], abi.PAIR))
        assert e.value.status == abi.DIO_ERR_INVALID


def test_zero_iterations_follow_reference_parities():
    sc = scenes.pyramid(levels=3)
    rows, off, idx = _avbd_inputs(sc)
    o = ph.avbd_options(iterations=0)
    ro = ph.run_options(o)
    args = (sc.state, sc.bodies["position"][:, :3], sc.bodies["orientation"], rows, sc.constraints, off, idx, ro)
    ref = O.avbd_run(*args)
    with compute.AvbdCompute(sc.n, max(64, len(rows))) as ac:
        got = ac.run(*args)
    for k in ref:
        assert np.array_equal(_bits(got[k]), _bits(ref[k])), k


def _gpu_pairs(bodies, hull=None, broad_phase=0):
    n = len(bodies)
    hv = hull if hull is not None else np.zeros((1, 4), np.float32)
    with compute.NarrowPhaseCompute(n, max(64, 64 * n), max_hull_vertices=len(hv)) as npc:
        npc.configure(broad_phase=broad_phase)
        npc.set_hull_vertices(hv)
        npc.submit_broad(bodies)
        c = npc.read_pair_count()
        return npc.read_pairs(c)


@pytest.mark.parametrize("broad_phase", [0, 1])
def test_lbvh_and_dense_pair_sets_at_scale(broad_phase):
    """The LBVH (default) and the dense sweep give the oracle's pair set in
    (a, b) order on larger scenes, including coincident and nested bodies."""
    cases = [scenes.cube_field(nx=16, nz=16, ny=4), scenes.mixed_pile(n=3000, extent=12.0)]
    # degenerate: many bodies at the same centre (equal Morton codes) plus a big one
    b, s = ph.pack_bodies([ph.sphere((0, 0, 0), 0.5, 1.0) for _ in range(40)] + [ph.cube((0, 0, 0), 5.0, 1.0)]
                          + [ph.sphere((20, 0, 0), 0.5, 1.0)])
    cases.append(scenes.Scene("coincident", b, s))
    for sc in cases:
        ref, _ = O.broad(sc.bodies, hull=sc.hull_vertices)
        got = _gpu_pairs(sc.bodies, sc.hull_vertices, broad_phase)
        assert np.array_equal(got, ref), sc.name


def test_world_with_large_and_small_scenes_matches_oracle():
    """Scenes up to the shared-memory tree size are refitted and traversed by
    one CTA each, larger ones by the global kernels; a world holding both
    (2304-body cube field between small scenes, LBVH rebuilt every 2 steps)
    still steps to the oracle's bits."""
    parts = [scenes.pyramid(levels=3), scenes.cube_field(nx=16, nz=16, ny=9), scenes.box_demo()]
    for p in parts:
        p.options = parts[0].options
    packed = scenes.pack(parts)
    ow = O.World(packed)
    ow.step(packed.options, 6)
    with _world(packed, bvh_rebuild_period=2) as w:
        w.step(packed.options, 6)
        gb, gs = w.download()
        gc = w.contacts()
        st = w.stats()
    rb, rs = ow.download()
    assert st["error_flags"] == 0 and st["pairs"] > 1000
    assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))
    assert np.array_equal(_bits(gc), _bits(ow.contacts()))


def _overlapping_field(n, seed):
    """n cubes and spheres (half size 0.5) on a 0.9 grid: neighbours overlap."""
    rng = np.random.default_rng(seed)
    side = int(np.ceil(n ** (1.0 / 3.0)))
    items = []
    for k in range(n):
        x, y, z = k % side, (k // side) % side, k // (side * side)
        p = (0.9 * x + rng.uniform(-0.05, 0.05), 0.5 + 0.9 * z, 0.9 * y + rng.uniform(-0.05, 0.05))
        items.append(ph.cube(p, 0.5, 1.0) if k % 3 else ph.sphere(p, 0.5, 1.0))
    b, st = ph.pack_bodies(items)
    return scenes.Scene(f"field{n}", b, st, containers=[scenes.ground()],
                        options=ph.avbd_options(gravity=(0, -9.81, 0), iterations=10))


def test_scene_tree_capacity_boundaries_match_oracle():
    """A scene of exactly the shared-memory tree's capacity (2048 bodies, one
    CTA), one of 2049 (the global kernels) and two scenes that fill one chunk
    exactly (1000 + 1048) step to the oracle's bits, LBVH rebuilt every 2 steps."""
    parts = [_overlapping_field(2048, 1), _overlapping_field(2049, 2), _overlapping_field(1000, 3),
             _overlapping_field(1048, 4)]
    packed = scenes.pack(parts)
    ow = O.World(packed)
    ow.step(packed.options, 3)
    with _world(packed, bvh_rebuild_period=2) as w:
        w.step(packed.options, 3)
        gb, gs = w.download()
        gc = w.contacts()
        st = w.stats()
    rb, rs = ow.download()
    assert st["error_flags"] == 0 and st["pairs"] > 10000
    assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))
    assert np.array_equal(_bits(gc), _bits(ow.contacts()))


@pytest.mark.parametrize("use_graph", [0, 1])
def test_profiled_world_times_every_primal_launch(use_graph):
    """With event timers on, every primal launch of the per-phase solve is
    timed, and every scene-chunk solve launch of the one-launch solve."""
    sc = scenes.box_demo()
    with _world(sc, use_graph=use_graph, profile=1, batched_solver=abi.SOLVE_PER_PHASE) as w:
        w.step(sc.options, 3)
        w.reset_timers()
        w.step(sc.options, 4)
        st = w.stats()
    iters = sc.options.iterations
    assert st["primal_launches"] == 4 * iters and st["chunk_launches"] == 0
    assert st["primal_ms"] > 0 and st["solve_ms"] >= st["primal_ms"]
    assert st["kernel_launches"] > 4 * 2 * iters
    with _world(sc, use_graph=use_graph, profile=1) as w:
        w.step(sc.options, 3)
        w.reset_timers()
        w.step(sc.options, 4)
        st = w.stats()
    assert st["chunk_launches"] == 4 and st["primal_launches"] == 0
    assert st["chunk_ms"] > 0 and st["solve_ms"] >= st["chunk_ms"]


def test_nonfinite_state_is_reported():
    """A NaN injected on the host (as a caller's bad input would arrive) is
    reported as DIO_ERR_NONFINITE after the step, not silently propagated."""
    sc = scenes.constraints_demo()
    with _world(sc) as w:
        w.step(sc.options, 2)
        b, s = w.download()
        bad = s.copy()
        bad["vel"][1, 0] = np.nan
        w.set_state(None, bad)
        with pytest.raises(abi.DioError) as e:
            w.step(sc.options, 1)
        assert e.value.status == abi.DIO_ERR_NONFINITE
        w.set_state(b, s)  # recovers once the state is finite again
        w.step(sc.options, 1)


def test_hull_pairs_with_staged_vertices_match_oracle():
    """EPA on hull pairs (vertices staged by bulk copies into shared memory)."""
    sc = scenes.mixed_pile(n=1500, extent=7.0, seed=11)
    pairs, _ = O.broad(sc.bodies, hull=sc.hull_vertices)
    ref = O.narrow(sc.bodies, pairs, hull=sc.hull_vertices)
    with compute.NarrowPhaseCompute(sc.n, len(pairs), max_hull_vertices=len(sc.hull_vertices)) as npc:
        npc.set_hull_vertices(sc.hull_vertices)
        got = npc.run(sc.bodies, pairs)
    assert int(ref["valid"].sum()) > 100
    assert np.array_equal(_bits(got), _bits(ref))


def _platform_scene():
    """A dynamic plate on the ground carrying a 4 x 4 grid of cubes: the plate
    has 16 x 4 contact rows plus its ground rows, over two 32-row rounds of
    the warp-per-body primal."""
    items = [ph.box((0.0, 0.1, 0.0), (2.2, 0.1, 2.2), 40.0)]
    for gx in range(4):
        for gz in range(4):
            items.append(ph.cube((-1.5 + gx * 1.0, 0.2 + 0.25 + 0.004, -1.5 + gz * 1.0), 0.25, 2.0))
    b, st = ph.pack_bodies(items)
    return scenes.Scene("platform", b, st, containers=[scenes.ground()], options=ph.avbd_options(), steps=8)


@pytest.mark.parametrize("variant", range(abi.PRIMAL_VARIANTS))
def test_every_primal_variant_matches_oracle(variant):
    """Launch shapes, tiles, per-position records, paired joint loads and the
    warp-per-body sums all compute the oracle's bits (joints of every kind,
    contacts, ground, a body with more than 64 rows); the per-phase solve is
    the one that runs the primal variants."""
    sc = scenes.pack([scenes.box_demo(), scenes.constraints_demo(), scenes.pyramid(levels=4), _platform_scene()])
    ow = O.World(sc)
    ow.step(sc.options, 8)
    with _world(sc, primal_variant=variant, batched_solver=abi.SOLVE_PER_PHASE) as w:
        w.step(sc.options, 8)
        gb, gs = w.download()
    rb, rs = ow.download()
    assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))


def _fib_sphere(n, r):
    k = np.arange(n) + 0.5
    phi = np.arccos(1 - 2 * k / n)
    th = np.pi * (1 + 5 ** 0.5) * k
    return (r * np.stack([np.cos(th) * np.sin(phi), np.sin(th) * np.sin(phi), np.cos(phi)], 1)).astype(np.float32)


def test_hulls_beyond_the_staging_area_match_oracle():
    """EPA on hulls of 150 vertices -- more than the 64 per hull staged in
    shared memory, so read from global memory -- next to staged 42-vertex
    icospheres and against each other."""
    big, small = _fib_sphere(150, 0.5), (scenes.icosphere42() * 0.4).astype(np.float32)
    rng = np.random.default_rng(3)
    items, hv, first = [], [], 0
    for k in range(60):
        verts = big if k % 2 == 0 else small
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        items.append(ph.hull(tuple(rng.uniform(-1.5, 1.5, 3)), first, verts, 1.0, orientation=tuple(q)))
        hv.append(verts)
        first += len(verts)
    b, _ = ph.pack_bodies(items)
    hvs = np.zeros((first, 4), np.float32)
    hvs[:, :3] = np.concatenate(hv)
    pairs, _ = O.broad(b, hull=hvs)
    ref = O.narrow(b, pairs, hull=hvs)
    with compute.NarrowPhaseCompute(len(b), len(pairs), max_hull_vertices=len(hvs)) as npc:
        npc.set_hull_vertices(hvs)
        got = npc.run(b, pairs)
    big_pairs = ((ref["a"] % 2 == 0) & (ref["b"] % 2 == 0) & (ref["valid"] != 0)).sum()
    assert int(ref["valid"].sum()) > 20 and big_pairs > 0
    assert np.array_equal(_bits(got), _bits(ref))


def test_autotune_keeps_state_and_results(tmp_path):
    """Every tuned variant computes the same bits, and the trials run from a
    snapshot that is restored: stepping after tuning still matches the
    oracle exactly; a second call reuses the cache file."""
    sc = scenes.pack([scenes.box_demo(), scenes.constraints_demo(), scenes.pyramid(levels=4)])
    ow = O.World(sc)
    ow.step(sc.options, 3)
    with _world(sc) as w:
        w.step(sc.options, 3)
        before = w.download()
        cache = str(tmp_path / "tune.txt")
        cfg = w.autotune(sc.options, trial_steps=2, cache_path=cache)
        after = w.download()
        assert np.array_equal(_bits(before[0]), _bits(after[0]))
        assert np.array_equal(_bits(before[1]), _bits(after[1]))
        assert 0 <= cfg["primal_variant"] < abi.PRIMAL_VARIANTS and cfg["bvh_rebuild_period"] >= 1
        cfg2 = w.autotune(sc.options, trial_steps=2, cache_path=cache)
        assert (cfg2["primal_variant"], cfg2["bvh_rebuild_period"]) == (cfg["primal_variant"],
                                                                        cfg["bvh_rebuild_period"])
        w.step(sc.options, 10)
        ow.step(sc.options, 10)
        gb, gs = w.download()
    rb, rs = ow.download()
    assert np.array_equal(_bits(gb), _bits(rb)) and np.array_equal(_bits(gs), _bits(rs))


def _independent(colors, rows, joints, dyn):
    for a, b in list(zip(rows["a"], rows["b"])) + list(zip(joints["a"], joints["b"])):
        if b == abi.CONTAINER or a == b or not (dyn[a] and dyn[b]):
            continue
        if colors[a] == colors[b]:
            return False
    return True


@pytest.mark.parametrize("batched_solver,use_graph,variant", [(abi.SOLVE_AUTO, 1, 0), (abi.SOLVE_AUTO, 0, 0),
                                                              (abi.SOLVE_PER_PHASE, 1, 0),
                                                              (abi.SOLVE_PER_PHASE, 1, 10)])
def test_colored_world_matches_oracle(batched_solver, use_graph, variant):
    """Coloured Gauss-Seidel mode: the colouring (Jones-Plassmann, hashed
    priorities) and the resulting states equal the oracle's bit for bit --
    colouring and per-colour sweeps inside the scene-chunk solve (one launch
    per step, graph-captured) and with the host-driven colour loop, with a
    thread or a warp per body in the sweeps."""
    parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo()]
    for p in parts:
        p.options = parts[0].options
    for sc in [scenes.pyramid(levels=5), scenes.constraints_demo(), scenes.box_demo(),
               scenes.cube_field(nx=6, nz=6, ny=3), scenes.pack(parts)]:
        ow = O.World(sc, solver_mode=1)
        with _world(sc, solver_mode=1, batched_solver=batched_solver, use_graph=use_graph,
                    primal_variant=variant) as w:
            for step in range(30):
                ow.step(sc.options, 1)
                w.step(sc.options, 1)
                gc, rc = w.colors(), ow.colors()
                assert np.array_equal(gc, rc), (sc.name, step)
            gb, gs = w.download()
            rows = w.contacts()
        rb, rs = ow.download()
        assert np.array_equal(_bits(gb), _bits(rb)), sc.name
        assert np.array_equal(_bits(gs), _bits(rs)), sc.name
        dyn = sc.state["inv_mass"] != 0
        assert _independent(gc, rows, sc.constraints, dyn), sc.name


def test_motion_records_round_trip_and_host_loop():
    """The per-frame motion records (pose and velocities, 64 B per body):
    a world stepped by dio_world_set_motion / dio_step / dio_world_download_motion
    equals the world stepped by set_state / dio_step / download; and
    dio_worlds_step_motion_host over three worlds on three streams gives,
    frame by frame, the bits of the packed world."""
    torch = pytest.importorskip("torch")
    parts = [scenes.pyramid(levels=3), scenes.constraints_demo(), scenes.box_demo(),
             scenes.mixed_pile(n=120, extent=3.0)]
    for p in parts:
        p.options = parts[0].options
    packed = scenes.pack(parts)
    frames = 4
    with _world(packed) as w:
        b, s = w.download()
        for _ in range(frames):
            w.set_state(b, s)
            w.step(packed.options, 1)
            b, s = w.download()
    with _world(packed) as w:
        m = w.download_motion()
        assert np.array_equal(m["position"], packed.bodies["position"][:, :3])
        for _ in range(frames):
            w.set_motion(m)
            w.step(packed.options, 1)
            m = w.download_motion()
        gb, gs = w.download()
    assert np.array_equal(_bits(gb), _bits(b)) and np.array_equal(_bits(gs), _bits(s))
    assert np.array_equal(m["position"], b["position"][:, :3]) and np.array_equal(m["orientation"], b["orientation"])
    assert np.array_equal(m["velocity"], s["vel"][:, :3]) and np.array_equal(m["prev_velocity"], s["prev_vel"][:, :3])
    groups, starts = packed.split(3)
    hm = torch.empty(packed.n * abi.MOTION.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(abi.MOTION)
    with _world(packed) as w0:
        hm[:] = w0.download_motion()
    streams = [torch.cuda.Stream() for _ in groups]
    worlds = [_world(g) for g in groups]
    try:
        for wg, st in zip(worlds, streams):
            wg.set_stream(st.cuda_stream)
        views = [hm[lo:lo + g.n] for g, lo in zip(groups, starts)]
        compute.step_motion_host(worlds, views, packed.options, frames)
        assert np.array_equal(hm["position"], b["position"][:, :3])
        assert np.array_equal(hm["angular_velocity"], s["ang"][:, :3])
    finally:
        for wg in worlds:
            wg.close()
