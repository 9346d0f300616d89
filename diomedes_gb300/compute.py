"""Context objects over the C ABI, mirroring the reference's compute objects.

  NarrowPhaseCompute  engine/src/render/compute.rs:149-735
  AvbdCompute         engine/src/render/gpu_physics.rs:196-684
  decode_contacts     engine/src/render/compute.rs:738-750
  World               the fused device-resident step (dio_world_* / dio_step)
Every call goes to libdio_cuda.so; a failing status raises abi.DioError.
"""
import ctypes

import numpy as np

from . import abi
from .abi import check, ptr


def capacity(max_bodies, max_pairs=None, max_contacts=None, max_joints=0, max_scenes=1, max_hull_vertices=0):
    c = abi.Capacity()
    c.max_bodies = max_bodies
    c.max_pairs = max_pairs if max_pairs is not None else max(16, 16 * max_bodies)
    c.max_contacts = max_contacts if max_contacts is not None else max(64, 4 * c.max_pairs + 24 * max_bodies)
    c.max_joints = max_joints
    c.max_scenes = max_scenes
    c.max_hull_vertices = max_hull_vertices
    return c


def check_hull_ranges(bodies, n_hull):
    """Host-side mirror of the library's upload check: every HULL body's
    vertex range [pad[0], pad[0] + pad[1]) lies inside a hull-vertex pool of
    n_hull vertices (the support queries and the EPA's bulk copies read it).
    Raises ValueError naming the first body that does not."""
    b = np.asarray(bodies)
    if not len(b):
        return
    sh = b["shape"]
    hull = sh["tag"] == abi.HULL
    end = sh["pad"][:, 0].astype(np.uint64) + sh["pad"][:, 1].astype(np.uint64)
    bad = np.flatnonzero(hull & (end > np.uint64(n_hull)))
    if len(bad):
        i = int(bad[0])
        raise ValueError(f"body {i}: hull vertices [{int(sh['pad'][i, 0])}, {int(end[i])}) lie beyond the "
                         f"{int(n_hull)}-vertex hull pool")


class Context:
    """Owns one DioCtx (a CUDA stream plus device buffers)."""

    def __init__(self, cap):
        L = abi.lib()
        h = ctypes.c_void_p()
        check(L.dio_ctx_create(ctypes.byref(cap), ctypes.byref(h)), None, "dio_ctx_create")
        self.h = h.value
        self.cap = cap
        self.L = L

    def close(self):
        if getattr(self, "h", None):
            self.L.dio_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def configure(self, **kw):
        c = abi.Config()
        check(self.L.dio_ctx_get_config(self.h, ctypes.byref(c)), self.h)
        for k, v in kw.items():
            setattr(c, k, v)
        check(self.L.dio_ctx_configure(self.h, ctypes.byref(c)), self.h, "dio_ctx_configure")
        return c

    def synchronize(self):
        check(self.L.dio_ctx_synchronize(self.h), self.h)


class NarrowPhaseCompute(Context):
    """NarrowPhaseCompute::{submit_broad, read_pair_count, read_pairs,
    submit, submit_narrow, read, run}."""

    def __init__(self, max_bodies, max_pairs, max_hull_vertices=0):
        super().__init__(capacity(max_bodies, max_pairs, max_contacts=max(64, max_pairs * 8),
                                  max_hull_vertices=max_hull_vertices))
        self.last_pairs = 0

    def set_hull_vertices(self, xyzw):
        xyzw = np.ascontiguousarray(xyzw, np.float32)
        check(self.L.dio_set_hull_vertices(self.h, ptr(xyzw), len(xyzw)), self.h)

    def submit_broad(self, bodies):
        bodies = np.ascontiguousarray(bodies, abi.BODY)
        check(self.L.dio_broad_submit(self.h, ptr(bodies), len(bodies)), self.h, "submit_broad")

    def read_pair_count(self):
        c = ctypes.c_uint32()
        check(self.L.dio_broad_pair_count(self.h, ctypes.byref(c)), self.h, "read_pair_count")
        return c.value

    def read_pairs(self, count):
        out = np.zeros(count, abi.PAIR)
        n = ctypes.c_uint32()
        check(self.L.dio_read_pairs(self.h, ptr(out), count, ctypes.byref(n)), self.h, "read_pairs")
        return out[: min(count, n.value)]

    def submit(self, bodies, pairs):
        bodies = np.ascontiguousarray(bodies, abi.BODY)
        pairs = np.ascontiguousarray(pairs, abi.PAIR)
        self.last_pairs = len(pairs)
        check(self.L.dio_narrow_submit_pairs(self.h, ptr(bodies), len(bodies), ptr(pairs), len(pairs)),
              self.h, "submit")

    def submit_narrow(self, pair_count):
        self.last_pairs = pair_count
        check(self.L.dio_narrow_submit(self.h, pair_count), self.h, "submit_narrow")

    def read(self, per_pair=abi.CONTACTS_PER_PAIR):
        out = np.zeros(self.last_pairs * per_pair, abi.CONTACT_OUT)
        n = ctypes.c_uint32()
        check(self.L.dio_narrow_read(self.h, ptr(out), len(out), ctypes.byref(n)), self.h, "read")
        return out[: n.value]

    def run(self, bodies, pairs):
        self.submit(bodies, pairs)
        return self.read()


def decode_contacts(raw):
    """decode_contacts, compute.rs:738-750: the valid slots in slot order."""
    return raw[raw["valid"] != 0]


class AvbdCompute(Context):
    """AvbdCompute::{submit, read, run} plus the device contact preparation
    (AvbdSolver::prepare_contacts)."""

    def __init__(self, max_bodies, max_contacts, max_joints=64, max_pairs=None):
        mp = max_pairs if max_pairs is not None else max(16, max_contacts)
        super().__init__(capacity(max_bodies, mp, max_contacts, max_joints=max_joints))
        self.last_n = 0
        self.last_m = 0

    def submit(self, state, positions, orientations, contacts, constraints, offsets, indices, run_options):
        state = np.ascontiguousarray(state, abi.BODY_STATE)
        positions = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
        orientations = np.ascontiguousarray(orientations, np.float32).reshape(-1, 4)
        contacts = np.ascontiguousarray(contacts, abi.CONTACT)
        constraints = np.ascontiguousarray(constraints, abi.CONSTRAINT)
        offsets = np.ascontiguousarray(offsets, np.uint32)
        indices = np.ascontiguousarray(indices, np.uint32)
        self.last_n, self.last_m = len(state), len(contacts)
        check(self.L.dio_avbd_submit(self.h, ptr(state), ptr(positions), ptr(orientations), len(state),
                                     ptr(contacts), len(contacts), ptr(constraints), len(constraints),
                                     ptr(offsets), ptr(indices), ctypes.byref(run_options)),
              self.h, "avbd submit")

    def read(self):
        n, m = self.last_n, self.last_m
        out = {
            "positions": np.zeros((n, 3), np.float32),
            "orientations": np.zeros((n, 4), np.float32),
            "velocities": np.zeros((n, 3), np.float32),
            "angular_velocities": np.zeros((n, 3), np.float32),
            "prev_velocities": np.zeros((n, 3), np.float32),
            "lambda": np.zeros((m, 3), np.float32),
            "penalty": np.zeros((m, 3), np.float32),
        }
        r = abi.AvbdResult(ptr(out["positions"]), ptr(out["orientations"]), ptr(out["velocities"]),
                           ptr(out["angular_velocities"]), ptr(out["prev_velocities"]), ptr(out["lambda"]),
                           ptr(out["penalty"]))
        check(self.L.dio_avbd_read(self.h, ctypes.byref(r)), self.h, "avbd read")
        return out

    def run(self, *args):
        self.submit(*args)
        return self.read()

    def prepare_contacts(self, bodies, state, slots, prev, container, options):
        bodies = np.ascontiguousarray(bodies, abi.BODY)
        state = np.ascontiguousarray(state, abi.BODY_STATE)
        slots = np.ascontiguousarray(slots, abi.CONTACT_OUT)
        prev = np.ascontiguousarray(prev if prev is not None else np.zeros(0, abi.CONTACT), abi.CONTACT)
        n = len(bodies)
        cap = int(self.cap.max_contacts)
        out = np.zeros(cap, abi.CONTACT)
        offsets = np.zeros(n + 1, np.uint32)
        indices = np.zeros(2 * cap, np.uint32)
        m = ctypes.c_uint32()
        cptr = ctypes.byref(container) if container is not None else None
        check(self.L.dio_prepare_contacts(self.h, ptr(bodies), ptr(state), n, ptr(slots), len(slots), ptr(prev),
                                          len(prev), cptr, ctypes.byref(options), ptr(out), cap, ctypes.byref(m),
                                          ptr(offsets), ptr(indices), len(indices)),
              self.h, "prepare_contacts")
        return out[: m.value].copy(), offsets, indices[: offsets[-1]].copy()


def step_motion_host(worlds, motions, options, steps=1):
    """dio_worlds_step_motion_host: the per-frame loop with motion records
    (abi.MOTION) over a batch held as several worlds (one per stream);
    motions[g] is world g's host array (page-locked for overlapped copies),
    updated in place; returns after every world has finished."""
    n = len(worlds)
    if len(motions) != n:
        raise ValueError("one motion array per world")
    for g in range(n):
        m = motions[g]
        if len(m) != worlds[g].n or m.dtype != abi.MOTION or not m.flags.c_contiguous:
            raise ValueError(f"world {g}: motion must be {worlds[g].n} contiguous abi.MOTION records")
    hs = (ctypes.c_void_p * n)(*[w.h for w in worlds])
    ms = (ctypes.c_void_p * n)(*[ptr(m) for m in motions])
    rc = abi.lib().dio_worlds_step_motion_host(hs, n, ms, ctypes.byref(options), steps)
    if rc != abi.DIO_OK:
        failed = next((w.h for w in worlds if abi.lib().dio_ctx_last_error(w.h)), None)
        check(rc, failed, "dio_worlds_step_motion_host")


def step_host(worlds, bodies, states, options, steps=1):
    """dio_worlds_step_host: the per-frame upload / step / read-back loop over
    a batch held as several worlds (one per stream).  bodies[g] / states[g]
    are world g's host arrays (page-locked for overlapped copies), updated in
    place; returns after every world has finished."""
    n = len(worlds)
    if not (len(bodies) == len(states) == n):
        raise ValueError("one bodies and one state array per world")
    for g in range(n):
        if len(bodies[g]) != worlds[g].n or len(states[g]) != worlds[g].n:
            raise ValueError(f"world {g}: arrays must hold {worlds[g].n} bodies")
        if not (bodies[g].flags.c_contiguous and states[g].flags.c_contiguous):
            raise ValueError(f"world {g}: arrays must be contiguous (updated in place)")
        if bodies[g].dtype != abi.BODY or states[g].dtype != abi.BODY_STATE:
            raise ValueError(f"world {g}: arrays must be abi.BODY and abi.BODY_STATE records")
    hs = (ctypes.c_void_p * n)(*[w.h for w in worlds])
    bp = (ctypes.c_void_p * n)(*[ptr(b) for b in bodies])
    sp = (ctypes.c_void_p * n)(*[ptr(s) for s in states])
    rc = abi.lib().dio_worlds_step_host(hs, n, bp, sp, ctypes.byref(options), steps)
    if rc != abi.DIO_OK:
        failed = next((w.h for w in worlds if abi.lib().dio_ctx_last_error(w.h)), None)
        check(rc, failed, "dio_worlds_step_host")


def checkpoint_header(image):
    """The header fields of a checkpoint image (abi.CKPT_HEADER)."""
    return np.frombuffer(image[: abi.CKPT_HEADER.itemsize], abi.CKPT_HEADER)[0]


class World(Context):
    """A device-resident world of one or more packed scenes (dio_world_*)."""

    def __init__(self, cap, **config):
        super().__init__(cap)
        if config:
            self.configure(**config)
        self.n = 0

    def upload(self, bodies, state, constraints=None, scene_offsets=None, containers=None, hull_vertices=None,
               positions_f64=None, orientations_f64=None):
        bodies = np.ascontiguousarray(bodies, abi.BODY)
        state = np.ascontiguousarray(state, abi.BODY_STATE)
        cons = np.ascontiguousarray(constraints if constraints is not None else np.zeros(0, abi.CONSTRAINT),
                                    abi.CONSTRAINT)
        d = abi.WorldDesc()
        d.n_bodies = len(bodies)
        d.n_constraints = len(cons)
        keep = [bodies, state, cons]
        d.bodies, d.state, d.constraints = ptr(bodies), ptr(state), ptr(cons)
        if scene_offsets is not None:
            so = np.ascontiguousarray(scene_offsets, np.uint32)
            keep.append(so)
            d.n_scenes = len(so) - 1
            d.scene_offsets = ptr(so)
        if containers is not None:
            if isinstance(containers, abi.Container):
                containers = [containers]
            arr = (abi.Container * len(containers))(*containers)
            keep.append(arr)
            d.containers = ctypes.addressof(arr)
            if scene_offsets is None:
                d.n_scenes = 1
        if hull_vertices is not None and len(hull_vertices):
            hv = np.ascontiguousarray(hull_vertices, np.float32).reshape(-1, 4)
            keep.append(hv)
            d.n_hull_vertices = len(hv)
            d.hull_vertices = ptr(hv)
        check_hull_ranges(bodies, d.n_hull_vertices)
        if positions_f64 is not None:
            p = np.ascontiguousarray(positions_f64, np.float64)
            keep.append(p)
            d.positions_f64 = ptr(p)
        if orientations_f64 is not None:
            q = np.ascontiguousarray(orientations_f64, np.float64)
            keep.append(q)
            d.orientations_f64 = ptr(q)
        check(self.L.dio_world_upload(self.h, ctypes.byref(d)), self.h, "world upload")
        self.n = len(bodies)

    def step(self, options, steps=1):
        check(self.L.dio_step(self.h, ctypes.byref(options), steps), self.h, "dio_step")

    def step_async(self, options, steps=1):
        """Enqueue steps without waiting; errors surface at synchronize()."""
        check(self.L.dio_step_async(self.h, ctypes.byref(options), steps), self.h, "dio_step_async")

    def download_async(self, bodies, state):
        """Enqueue the copy of poses / state into caller buffers (pinned for overlap)."""
        check(self.L.dio_world_download_async(self.h, ptr(bodies), ptr(state)), self.h, "download_async")

    def set_stream(self, cuda_stream_handle):
        check(self.L.dio_ctx_set_stream(self.h, cuda_stream_handle), self.h, "set_stream")

    def set_state(self, bodies=None, state=None):
        b = None if bodies is None else np.ascontiguousarray(bodies, abi.BODY)
        s = None if state is None else np.ascontiguousarray(state, abi.BODY_STATE)
        check(self.L.dio_world_set_state(self.h, ptr(b), ptr(s)), self.h, "set_state")

    def set_motion(self, motion):
        """dio_world_set_motion: poses and velocities (abi.MOTION records)."""
        m = np.ascontiguousarray(motion, abi.MOTION)
        if len(m) != self.n:
            raise ValueError(f"motion records must hold {self.n} bodies")
        check(self.L.dio_world_set_motion(self.h, ptr(m)), self.h, "set_motion")

    def download_motion_into(self, motion):
        if len(motion) != self.n or motion.dtype != abi.MOTION or not motion.flags.c_contiguous:
            raise ValueError(f"motion records must be {self.n} contiguous abi.MOTION records")
        check(self.L.dio_world_download_motion(self.h, ptr(motion)), self.h, "download_motion")

    def download_motion(self):
        m = np.zeros(self.n, abi.MOTION)
        self.download_motion_into(m)
        return m

    def download_into(self, bodies, state):
        check(self.L.dio_world_download(self.h, ptr(bodies), ptr(state)), self.h, "download")

    def download(self):
        b = np.zeros(self.n, abi.BODY)
        s = np.zeros(self.n, abi.BODY_STATE)
        check(self.L.dio_world_download(self.h, ptr(b), ptr(s)), self.h, "download")
        return b, s

    def download_f64(self):
        p = np.zeros((self.n, 3), np.float64)
        q = np.zeros((self.n, 4), np.float64)
        check(self.L.dio_world_download_f64(self.h, ptr(p), ptr(q)), self.h, "download_f64")
        return p, q

    def contacts(self):
        m = ctypes.c_uint32()
        cap = int(self.cap.max_contacts)
        out = np.zeros(cap, abi.CONTACT)
        check(self.L.dio_world_contacts(self.h, ptr(out), cap, ctypes.byref(m)), self.h, "contacts")
        return out[: m.value].copy()

    def colors(self):
        out = np.zeros(self.n, np.uint32)
        n = ctypes.c_uint32()
        check(self.L.dio_world_colors(self.h, ptr(out), len(out), ctypes.byref(n)), self.h, "colors")
        return out

    def stats(self):
        s = abi.StepStats()
        check(self.L.dio_world_stats(self.h, ctypes.byref(s)), self.h, "stats")
        return {"pairs": s.pairs, "contacts": s.contacts, "colors": s.colors, "error_flags": s.error_flags,
                "steps": s.steps, "kernel_launches": s.kernel_launches, "primal_launches": s.primal_launches,
                "dual_launches": s.dual_launches, "primal_ms": s.primal_ms, "dual_ms": s.dual_ms,
                "broad_ms": s.broad_ms, "narrow_ms": s.narrow_ms, "rows_ms": s.rows_ms, "solve_ms": s.solve_ms,
                "chunk_launches": s.chunk_launches, "chunk_ms": s.chunk_ms}

    def autotune(self, options, trial_steps=5, cache_path=None):
        """dio_autotune: pick the fastest launch shape / LBVH rebuild period
        for this world (state unchanged); returns the chosen config."""
        c = abi.Config()
        path = cache_path.encode() if cache_path else None
        check(self.L.dio_autotune(self.h, ctypes.byref(options), trial_steps, path, ctypes.byref(c)), self.h,
              "autotune")
        return {name: getattr(c, name) for name, _ in abi.Config._fields_}

    def reset_timers(self):
        check(self.L.dio_world_reset_timers(self.h), self.h, "reset_timers")

    def export_transforms(self, out_ptr, stride, fmt=abi.XFORM_POSE, scales_ptr=None):
        """Write every body's transform into a device buffer (stream-ordered)."""
        check(self.L.dio_world_export_transforms(self.h, fmt, scales_ptr, out_ptr, stride), self.h,
              "export_transforms")

    def checkpoint(self):
        """The world as a versioned byte image (dio_world_checkpoint)."""
        size = ctypes.c_size_t()
        check(self.L.dio_world_checkpoint(self.h, None, 0, ctypes.byref(size)), self.h, "checkpoint")
        buf = np.zeros(size.value, np.uint8)
        check(self.L.dio_world_checkpoint(self.h, ptr(buf), size.value, ctypes.byref(size)), self.h, "checkpoint")
        return buf.tobytes()

    def resume(self, image):
        """Replace this context's world with a checkpoint image (dio_world_resume)."""
        buf = np.frombuffer(image, np.uint8)
        check(self.L.dio_world_resume(self.h, ptr(buf), buf.size), self.h, "resume")
        self.n = int(checkpoint_header(image)["n"])


def device_exclusive_scan(values, repeats=1, live=None, out=None):
    """Exclusive prefix sum of a uint32 array by the pipeline's device scan
    (uint32 wrap-around), run `repeats` times on the same buffers.  With
    `live`, only the first `live` entries are scanned (the count is handed
    over in device memory); the rest of `out` keeps its contents.  Returns
    (prefix sums, total of the live entries)."""
    a = np.ascontiguousarray(values, dtype=np.uint32)
    res = np.zeros_like(a) if out is None else np.array(out, dtype=np.uint32, copy=True)
    total = ctypes.c_uint32(0)
    n_live = a.size if live is None else live
    check(abi.lib().dio_selftest_scan(ptr(a), ptr(res), a.size, n_live, repeats, ctypes.byref(total)))
    return res, total.value


def device_sort_pairs(keys, values, begin_bit=0, end_bit=None):
    """Stable sort of (keys, values) by key bits [begin_bit, end_bit) with the
    pipeline's device radix sort; keys uint32 or uint64, values uint32."""
    k = np.ascontiguousarray(keys)
    if k.dtype not in (np.uint32, np.uint64):
        raise TypeError("keys must be uint32 or uint64")
    v = np.ascontiguousarray(values, dtype=np.uint32)
    if v.shape != k.shape:
        raise ValueError("keys and values differ in length")
    if end_bit is None:
        end_bit = 8 * k.dtype.itemsize
    ko, vo = np.empty_like(k), np.empty_like(v)
    fn = abi.lib().dio_selftest_sort_u64 if k.dtype == np.uint64 else abi.lib().dio_selftest_sort_u32
    check(fn(ptr(k), ptr(v), k.size, begin_bit, end_bit, ptr(ko), ptr(vo)))
    return ko, vo
