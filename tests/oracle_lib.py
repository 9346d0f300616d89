"""ctypes wrapper of the CPU oracle (oracle/liboracle.so) for the tests.

Tests feed the oracle the same records they feed the CUDA library and
compare the results.
"""
import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from diomedes_gb300 import abi  # noqa: E402

_u32 = ctypes.c_uint32
_vp = ctypes.c_void_p
_LIBS = {}


def lib(variant=""):
    """The oracle library; `variant` names a build variant of oracle/build.py
    (the default is the reference arithmetic)."""
    if variant not in _LIBS:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import build as oracle_build  # oracle/build.py

        path = oracle_build.build(variant=variant)
        L = ctypes.CDLL(path)
        protos = {
            "oracle_support": [_vp, _vp, _vp, _u32, _vp],
            "oracle_aabb": [_vp, _u32, _vp, _u32, _vp],
            "oracle_broad": [_vp, _u32, _vp, _u32, _u32, _vp, _u32, ctypes.POINTER(_u32)],
            "oracle_narrow": [_vp, _u32, _vp, _u32, _vp, _u32, _u32, _vp],
            "oracle_prepare_contacts": [_vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp,
                                        ctypes.POINTER(abi.AvbdOptions), _vp, _u32, _vp, _u32, ctypes.POINTER(_u32),
                                        _vp, _vp, _u32, ctypes.POINTER(_u32)],
            "oracle_avbd_run": [_u32, _vp, _vp, _vp, _u32, _vp, _u32, _vp, _u32, _vp, _vp,
                                ctypes.POINTER(abi.RunOptions), _u32, _vp, _vp, _vp, _vp, _vp, _vp, _vp],
            "oracle_world_step": [_vp, ctypes.POINTER(abi.AvbdOptions), _u32],
            "oracle_world_set_lag": [_vp, ctypes.c_int],
            "oracle_world_download": [_vp, _vp, _vp],
            "oracle_world_download_f64": [_vp, _vp, _vp],
            "oracle_world_contacts": [_vp, _vp, _u32, ctypes.POINTER(_u32)],
            "oracle_world_colors": [_vp, _vp, _u32, ctypes.POINTER(_u32)],
            "oracle_world_stats": [_vp, ctypes.POINTER(abi.StepStats)],
        }
        for k, a in protos.items():
            getattr(L, k).argtypes = a
            getattr(L, k).restype = ctypes.c_int
        L.oracle_world_create.argtypes = [ctypes.POINTER(abi.WorldDesc), ctypes.POINTER(abi.Config), ctypes.c_int]
        L.oracle_world_create.restype = _vp
        L.oracle_world_destroy.argtypes = [_vp]
        L.oracle_world_destroy.restype = None
        L.oracle_color_hash.argtypes = [_u32]
        L.oracle_color_hash.restype = _u32
        _LIBS[variant] = L
    return _LIBS[variant]


P = abi.ptr


def support(shape, d, hull=None):
    s = np.ascontiguousarray(np.asarray(shape, abi.SHAPE).reshape(1))
    d = np.ascontiguousarray(d, np.float32)
    h = np.zeros((0, 4), np.float32) if hull is None else np.ascontiguousarray(hull, np.float32)
    out = np.zeros(3, np.float32)
    lib().oracle_support(P(s), P(d), P(h), len(h), P(out))
    return out


def aabb(bodies, hull=None):
    b = np.ascontiguousarray(bodies, abi.BODY)
    h = np.zeros((0, 4), np.float32) if hull is None else np.ascontiguousarray(hull, np.float32)
    out = np.zeros((len(b), 8), np.float32)
    lib().oracle_aabb(P(b), len(b), P(h), len(h), P(out))
    return out


def broad(bodies, hull=None, sap=False, cap=None):
    b = np.ascontiguousarray(bodies, abi.BODY)
    h = np.zeros((0, 4), np.float32) if hull is None else np.ascontiguousarray(hull, np.float32)
    cap = cap if cap is not None else max(16, len(b) * 64)
    out = np.zeros(cap, abi.PAIR)
    n = _u32()
    lib().oracle_broad(P(b), len(b), P(h), len(h), int(sap), P(out), cap, ctypes.byref(n))
    return out[: min(cap, n.value)], n.value


def narrow(bodies, pairs, hull=None, per_pair=4):
    b = np.ascontiguousarray(bodies, abi.BODY)
    p = np.ascontiguousarray(pairs, abi.PAIR)
    h = np.zeros((0, 4), np.float32) if hull is None else np.ascontiguousarray(hull, np.float32)
    out = np.zeros(len(p) * per_pair, abi.CONTACT_OUT)
    lib().oracle_narrow(P(b), len(b), P(p), len(p), P(h), len(h), per_pair, P(out))
    return out


def prepare_contacts(bodies, state, slots, prev, container, options, hull=None):
    b = np.ascontiguousarray(bodies, abi.BODY)
    s = np.ascontiguousarray(state, abi.BODY_STATE)
    sl = np.ascontiguousarray(slots, abi.CONTACT_OUT)
    pv = np.ascontiguousarray(prev if prev is not None else np.zeros(0, abi.CONTACT), abi.CONTACT)
    h = np.zeros((0, 4), np.float32) if hull is None else np.ascontiguousarray(hull, np.float32)
    n = len(b)
    cap = len(sl) + 24 * n + 16
    out = np.zeros(cap, abi.CONTACT)
    off = np.zeros(n + 1, np.uint32)
    idx = np.zeros(2 * cap, np.uint32)
    m, ni = _u32(), _u32()
    cptr = ctypes.byref(container) if container is not None else None
    rc = lib().oracle_prepare_contacts(P(b), P(s), n, P(sl), len(sl), P(pv), len(pv), cptr, ctypes.byref(options),
                                       P(h), len(h), P(out), cap, ctypes.byref(m), P(off), P(idx), len(idx),
                                       ctypes.byref(ni))
    assert rc == 0, rc
    return out[: m.value].copy(), off, idx[: ni.value].copy()


def avbd_run(state, positions, orientations, contacts, constraints, offsets, indices, run_options, precision=0,
             joint_csr=False):
    st = np.ascontiguousarray(state, abi.BODY_STATE)
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 3)
    q = np.ascontiguousarray(orientations, np.float32).reshape(-1, 4)
    c = np.ascontiguousarray(contacts, abi.CONTACT)
    j = np.ascontiguousarray(constraints, abi.CONSTRAINT)
    off = np.ascontiguousarray(offsets, np.uint32)
    idx = np.ascontiguousarray(indices, np.uint32)
    n, m = len(st), len(c)
    out = {
        "positions": np.zeros((n, 3), np.float32),
        "orientations": np.zeros((n, 4), np.float32),
        "velocities": np.zeros((n, 3), np.float32),
        "angular_velocities": np.zeros((n, 3), np.float32),
        "prev_velocities": np.zeros((n, 3), np.float32),
        "lambda": np.zeros((m, 3), np.float32),
        "penalty": np.zeros((m, 3), np.float32),
    }
    lib().oracle_avbd_run(precision, P(st), P(pos), P(q), n, P(c), m, P(j), len(j), P(off), P(idx),
                          ctypes.byref(run_options), int(joint_csr), P(out["positions"]), P(out["orientations"]),
                          P(out["velocities"]), P(out["angular_velocities"]), P(out["prev_velocities"]),
                          P(out["lambda"]), P(out["penalty"]))
    return out


class World:
    """Oracle world: same descriptor as the CUDA world."""

    def __init__(self, scene, precision=0, solver_mode=0, contacts_per_pair=4, threads=1, contact_lag=0,
                 variant=""):
        self._keep = []
        self.L = lib(variant)
        d = abi.WorldDesc()
        b = np.ascontiguousarray(scene.bodies, abi.BODY)
        s = np.ascontiguousarray(scene.state, abi.BODY_STATE)
        c = np.ascontiguousarray(scene.constraints, abi.CONSTRAINT)
        self._keep += [b, s, c]
        d.n_bodies, d.n_constraints = len(b), len(c)
        d.bodies, d.state, d.constraints = P(b), P(s), P(c)
        if scene.scene_offsets is not None:
            so = np.ascontiguousarray(scene.scene_offsets, np.uint32)
            self._keep.append(so)
            d.n_scenes = len(so) - 1
            d.scene_offsets = P(so)
        if scene.containers:
            arr = (abi.Container * len(scene.containers))(*scene.containers)
            self._keep.append(arr)
            d.containers = ctypes.addressof(arr)
            if scene.scene_offsets is None:
                d.n_scenes = 1
        if scene.hull_vertices is not None and len(scene.hull_vertices):
            hv = np.ascontiguousarray(scene.hull_vertices, np.float32)
            self._keep.append(hv)
            d.n_hull_vertices = len(hv)
            d.hull_vertices = P(hv)
        if scene.positions_f64 is not None:
            p64 = np.ascontiguousarray(scene.positions_f64, np.float64)
            self._keep.append(p64)
            d.positions_f64 = P(p64)
        cfg = abi.Config()
        cfg.precision = precision
        cfg.solver_mode = solver_mode
        cfg.contacts_per_pair = contacts_per_pair
        cfg.contact_lag = contact_lag
        self.h = self.L.oracle_world_create(ctypes.byref(d), ctypes.byref(cfg), threads)
        self.n = len(b)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_world_destroy(self.h)
            self.h = None

    def step(self, options, steps=1):
        self.L.oracle_world_step(self.h, ctypes.byref(options), steps)

    def set_lag(self, on):
        self.L.oracle_world_set_lag(self.h, int(on))

    def download(self):
        b = np.zeros(self.n, abi.BODY)
        s = np.zeros(self.n, abi.BODY_STATE)
        self.L.oracle_world_download(self.h, P(b), P(s))
        return b, s

    def download_f64(self):
        p = np.zeros((self.n, 3), np.float64)
        q = np.zeros((self.n, 4), np.float64)
        self.L.oracle_world_download_f64(self.h, P(p), P(q))
        return p, q

    def contacts(self):
        m = _u32()
        self.L.oracle_world_contacts(self.h, None, 0, ctypes.byref(m))
        out = np.zeros(max(1, m.value), abi.CONTACT)
        self.L.oracle_world_contacts(self.h, P(out), len(out), ctypes.byref(m))
        return out[: m.value]

    def colors(self):
        out = np.zeros(self.n, np.uint32)
        n = _u32()
        self.L.oracle_world_colors(self.h, P(out), len(out), ctypes.byref(n))
        return out[: n.value]

    def stats(self):
        s = abi.StepStats()
        self.L.oracle_world_stats(self.h, ctypes.byref(s))
        return {"pairs": s.pairs, "contacts": s.contacts, "colors": s.colors, "error_flags": s.error_flags}
