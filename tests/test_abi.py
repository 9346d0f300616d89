"""CPU checks of the boundary: the library loads, exports every symbol the
header declares, and the record layouts match the reference's byte sizes."""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

from diomedes_gb300 import abi, physics as ph

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in ("dio_cuda.h", "dio_selftest.h")]


def _declared():
    text = "".join(open(h).read() for h in HEADERS)
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(dio_\w+)\(", text, re.M)))


@pytest.fixture(scope="module")
def library():
    if not os.path.exists(abi.LIB_PATH):
        from diomedes_gb300 import build

        build.build()
    return ctypes.CDLL(abi.LIB_PATH)


def test_library_exports_every_declared_symbol(library):
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(library, n), n
    # and the ctypes table covers the whole header
    assert set(names) == set(abi._PROTOS), set(names) ^ set(abi._PROTOS)


def test_exported_symbols_are_plain_c(library):
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    for n in _declared():
        assert n in exported, n  # unmangled extern "C"


def test_record_sizes_match_the_reference_layouts():
    # compute.rs GpuShape 80, GpuBody 112, GpuPair 8, GpuContactOut 80;
    # gpu_physics.rs GpuAvbdBodyState 80, GpuAvbdContact 144, GpuAvbdConstraint 48
    assert [abi.SHAPE.itemsize, abi.BODY.itemsize, abi.PAIR.itemsize, abi.CONTACT_OUT.itemsize] == [80, 112, 8, 80]
    assert [abi.BODY_STATE.itemsize, abi.CONTACT.itemsize, abi.CONSTRAINT.itemsize] == [80, 144, 48]
    assert ctypes.sizeof(abi.RunOptions) == 32 and ctypes.sizeof(abi.AvbdOptions) == 48


def test_body_constructors_follow_the_reference():
    b, s = ph.sphere((0, 0, 0), 0.3, 1.0)
    assert s["inv_mass"] == np.float32(1.0)
    assert s["inv_moment"][0] == np.float32(1.0) / (np.float32(0.4) * np.float32(1.0) * np.float32(0.3) * np.float32(0.3))
    b, s = ph.cube((0, 0, 0), 0.5, 2.0)
    assert b["shape"]["tag"] == abi.CUBE and b["shape"]["corners"][0, :3].tolist() == [0.5, 0.5, 0.5]
    assert s["friction"] == np.float32(0.8)
    b, s = ph.cube((0, 0, 0), 0.5, 0.0)
    assert s["inv_mass"] == 0 and (s["inv_moment"] == 0).all()


def test_default_options_match_avbd_options_default():
    o = ph.avbd_options()
    assert (o.iterations, round(o.alpha, 6), o.beta_lin, round(o.margin, 6), o.penalty_min) == (10, 0.99, 1e4, 0.01, 1.0)
    assert list(o.gravity) == [0.0, -10.0, 0.0]


def test_header_constants_match_the_python_mirror():
    with open(os.path.join(ROOT, "include", "dio_cuda.h")) as f:
        text = f.read()
    m = re.search(r"#define DIO_PRIMAL_VARIANTS (\d+)", text)
    assert m and int(m.group(1)) == abi.PRIMAL_VARIANTS
    m = re.search(r"DIO_XFORM_POSE = (\d+), DIO_XFORM_MAT4 = (\d+)", text)
    assert m and (int(m.group(1)), int(m.group(2))) == (abi.XFORM_POSE, abi.XFORM_MAT4)
    for name in ("DIO_OK", "DIO_ERR_INVALID", "DIO_ERR_CAPACITY", "DIO_ERR_TIMEOUT", "DIO_ERR_CUDA",
                 "DIO_ERR_NONFINITE", "DIO_ERR_STATE"):
        m = re.search(name + r"\s*=\s*(\d+)", text)
        assert m and int(m.group(1)) == getattr(abi, name), name


def test_bad_arguments_are_rejected_before_any_device_work():
    """Argument checks run before the library touches CUDA, so they hold on a
    machine without a GPU: null contexts and null outputs are DIO_ERR_INVALID,
    and the multi-world host loop rejects missing arrays (count 0 is a no-op)."""
    L = abi.lib()
    o = ph.avbd_options()
    assert L.dio_step(None, ctypes.byref(o), 1) == abi.DIO_ERR_INVALID
    assert L.dio_step_async(None, ctypes.byref(o), 1) == abi.DIO_ERR_INVALID
    assert L.dio_world_set_state(None, None, None) == abi.DIO_ERR_INVALID
    assert L.dio_world_download(None, None, None) == abi.DIO_ERR_INVALID
    assert L.dio_world_download_async(None, None, None) == abi.DIO_ERR_INVALID
    assert L.dio_ctx_synchronize(None) == abi.DIO_ERR_INVALID
    assert L.dio_world_checkpoint(None, None, 0, None) == abi.DIO_ERR_INVALID
    assert L.dio_world_resume(None, None, 0) == abi.DIO_ERR_INVALID
    assert L.dio_worlds_step_host(None, 0, None, None, ctypes.byref(o), 1) == abi.DIO_OK
    assert L.dio_worlds_step_host(None, 1, None, None, ctypes.byref(o), 1) == abi.DIO_ERR_INVALID
    one = (ctypes.c_void_p * 1)(None)
    assert L.dio_worlds_step_host(one, 1, one, one, ctypes.byref(o), 1) == abi.DIO_ERR_INVALID
    assert L.dio_worlds_step_host(one, 1, one, one, None, 1) == abi.DIO_ERR_INVALID
    assert L.dio_world_set_motion(None, None) == abi.DIO_ERR_INVALID
    assert L.dio_world_download_motion(None, None) == abi.DIO_ERR_INVALID
    assert L.dio_world_download_motion_async(None, None) == abi.DIO_ERR_INVALID
    assert L.dio_worlds_step_motion_host(None, 0, None, ctypes.byref(o), 1) == abi.DIO_OK
    assert L.dio_worlds_step_motion_host(one, 1, one, ctypes.byref(o), 1) == abi.DIO_ERR_INVALID
    assert abi.MOTION.itemsize == 64


def test_context_creation_without_a_device_fails_loudly():
    """No CPU fallback: without a CUDA device the context cannot be created
    and the Python wrapper raises."""
    from diomedes_gb300 import compute

    L = abi.lib()
    h = ctypes.c_void_p()
    rc = L.dio_ctx_create(ctypes.byref(compute.capacity(16)), ctypes.byref(h))
    if rc == abi.DIO_OK:  # a GPU is present: nothing to check here
        L.dio_ctx_destroy(h)
        pytest.skip("a CUDA device is present")
    assert rc == abi.DIO_ERR_CUDA and not h.value
    with pytest.raises(abi.DioError):
        compute.World(compute.capacity(16))


def test_step_host_checks_its_arrays_before_calling_the_library():
    """compute.step_host validates every world's host arrays (count, length,
    contiguity, record type) before anything reaches the C ABI."""
    from diomedes_gb300 import compute

    class World4:  # stands in for a world of 4 bodies; never reaches the library
        n = 4
        h = None

    o = ph.avbd_options()
    b, s = np.zeros(4, abi.BODY), np.zeros(4, abi.BODY_STATE)
    with pytest.raises(ValueError):
        compute.step_host([World4()], [b], [], o)
    with pytest.raises(ValueError):
        compute.step_host([World4()], [b[:3]], [s[:3]], o)
    with pytest.raises(ValueError):
        compute.step_host([World4()], [np.zeros(8, abi.BODY)[::2]], [s], o)
    with pytest.raises(ValueError):
        compute.step_host([World4()], [np.zeros(4, abi.BODY_STATE)], [s], o)


def test_hull_ranges_are_checked_on_the_host():
    """compute.check_hull_ranges mirrors the library's upload check: a HULL
    body's vertex range must lie inside the hull-vertex pool (including a
    first + count that wraps 32 bits)."""
    from diomedes_gb300 import compute, scenes

    sc = scenes.mixed_pile(n=60, extent=3.0)
    nh = len(sc.hull_vertices)
    compute.check_hull_ranges(sc.bodies, nh)
    b = sc.bodies.copy()
    i = int(np.flatnonzero(b["shape"]["tag"] == abi.HULL)[0])
    b["shape"]["pad"][i, 0] = nh - 1
    with pytest.raises(ValueError):
        compute.check_hull_ranges(b, nh)
    b["shape"]["pad"][i, 0] = 0xFFFFFFFF
    with pytest.raises(ValueError):
        compute.check_hull_ranges(b, nh)
    b["shape"]["pad"][i, 0] = nh - b["shape"]["pad"][i, 1]  # ends exactly at the pool end
    compute.check_hull_ranges(b, nh)
    with pytest.raises(ValueError):
        compute.check_hull_ranges(b, nh - 1)


def test_no_library_code_in_the_scans_and_sorts():
    # the prefix sums and radix sorts are the library's own kernels (k_scan.cuh)
    out = subprocess.run(["nm", "-C", abi.LIB_PATH], capture_output=True, text=True).stdout
    assert "cub::" not in out
    assert "dio::k_scan_excl" in out and "dio::k_radix_pass" in out
