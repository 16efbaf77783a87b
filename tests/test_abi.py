"""The C ABI library builds for sm_103a, loads, and exports every entry point
that include/krr_gb300.h declares (no GPU needed)."""
import re
import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "krr_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(krr_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_pass_interface():
    names = declared_functions()
    for n in ("krr_wf_create", "krr_wf_set_scene", "krr_wf_resize", "krr_wf_begin_frame",
              "krr_wf_render", "krr_accel_trace_closest", "krr_accel_trace_any"):
        assert n in names


def test_library_exports_every_declared_symbol(krr_lib):
    from kiraray_gb300 import _lib
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (krr_[a-z0-9_]+)$", out, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, f"declared but not exported: {missing}"


def test_binding_covers_every_declared_symbol(krr_lib):
    from kiraray_gb300 import _lib
    assert set(declared_functions()) <= set(_lib.SIGNATURES)
    for n in declared_functions():
        getattr(krr_lib, n)


def test_status_strings(krr_lib):
    assert krr_lib.krr_status_string(0) == b"ok"
    assert krr_lib.krr_status_string(3) == b"capacity overflow"
    assert krr_lib.krr_version() >= 1


def test_invalid_arguments_fail_without_gpu_work(krr_lib):
    import ctypes as C
    from kiraray_gb300 import _lib
    h = C.c_void_p()
    assert krr_lib.krr_accel_create_from_triangles(None, 5, C.byref(h), None) == 1
    assert krr_lib.krr_wf_create(None, None) == 1
    p = _lib.WfParams()
    krr_lib.krr_wf_params_default(C.byref(p))
    assert p.nee == 1 and p.max_depth == 10 and abs(p.rr - 0.8) < 1e-7 and p.clamp_max == 1e3
    # refit, rebuild and the BVH settings check their arguments before any GPU work
    assert krr_lib.krr_accel_refit_triangles(None, None, 0, None) == 1
    assert krr_lib.krr_wf_rebuild_bvh(None, None) == 1
    assert krr_lib.krr_wf_update_instances(None, 0, None, None, None) == 1
    for bad in (0, 4, -1):
        assert krr_lib.krr_set_bvh_max_leaf(bad) == 1
        assert krr_lib.krr_set_bvh_full_node_leaf(bad) == 1
    assert krr_lib.krr_set_bvh_node_format(2) == 1
    assert krr_lib.krr_set_bvh_treelets(4) == 1 and krr_lib.krr_set_bvh_treelets(-1) == 1
    assert krr_lib.krr_wf_set_camera_order(None, 1) == 1
    assert krr_lib.krr_wf_set_profiling(None, 1) == 1
    assert krr_lib.krr_wf_profile_read(None, None, 0, None) == 1
