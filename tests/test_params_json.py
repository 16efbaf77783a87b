"""Pass parameters from JSON through the C ABI (krr_wf_params_from_json /
krr_wf_create_json), host code only: the reference's from_json keys and
defaults (src/render/wavefront/integrator.h:85-103)."""
import ctypes as C

import pytest

from kiraray_gb300 import _lib


def _parse(text):
    lib = _lib.load()
    p = _lib.WfParams()
    st = lib.krr_wf_params_from_json(text.encode(), C.byref(p))
    return st, p


def test_defaults_and_every_key(krr_lib):
    st, p = _parse("{}")
    assert st == 0
    assert (p.nee, p.enable_medium, p.max_depth, p.enable_clamp, p.spp, p.seed) == (1, 1, 10, 0, 1, 0)
    assert p.rr == pytest.approx(0.8) and p.clamp_max == pytest.approx(1e3)
    st, p = _parse(' { "nee": false, "enable_medium": false, "max_depth": 6, "rr": 0.5,\n'
                   '   "enable_clamp": true, "clamp_max": 2.5e1, "spp": 4, "seed": 4000000000,'
                   '   "independent_samples": 1 } ')
    assert st == 0
    assert (p.nee, p.enable_medium, p.max_depth, p.enable_clamp, p.spp, p.seed,
            p.independent_samples) == (0, 0, 6, 1, 4, 4000000000, 1)
    assert p.rr == pytest.approx(0.5) and p.clamp_max == pytest.approx(25.0)


def test_other_keys_and_nested_values_are_skipped(krr_lib):
    st, p = _parse('{"name": "WavefrontPathTracer", "extra": {"a": [1, 2, {"b": null}], "s": "x\\"y"},'
                   ' "max_depth": 3, "list": [], "u": "\\u00e9"}')
    assert st == 0 and p.max_depth == 3 and p.nee == 1


@pytest.mark.parametrize("text", ['{"max_depth": "5"}', '{"max_depth": 2.5}', '{"nee": 3}',
                                  '{"rr": true}', '{"seed": -1}', '{"spp": 0}',
                                  '{"max_depth": -1}'])
def test_wrong_types_and_values_are_rejected(krr_lib, text):
    st, _ = _parse(text)
    assert st == 1   # KRR_ERR_INVALID_ARGUMENT
    assert _lib.load().krr_last_error()


@pytest.mark.parametrize("text", ["", "[]", "{", '{"nee": tru}', '{"nee" true}', '{"a": 1,}',
                                  '{"a": 01}', '{"a": 1} x', '{"a": "unterminated}', "{'a': 1}"])
def test_malformed_json_is_rejected(krr_lib, text):
    st, _ = _parse(text)
    assert st == 1


def test_create_from_json(krr_lib):
    lib = _lib.load()
    h = C.c_void_p()
    assert lib.krr_wf_create_json(b'{"max_depth": 7, "nee": false}', C.byref(h)) == 0
    p = _lib.WfParams()
    assert lib.krr_wf_get_params(h, C.byref(p)) == 0
    assert p.max_depth == 7 and p.nee == 0 and p.rr == pytest.approx(0.8)
    assert lib.krr_wf_set_params_json(h, b'{"rr": 0.25}') == 0
    assert lib.krr_wf_get_params(h, C.byref(p)) == 0
    assert p.max_depth == 7 and p.rr == pytest.approx(0.25)
    assert lib.krr_wf_set_params_json(h, b'{"rr": "x"}') == 1
    assert lib.krr_wf_get_params(h, C.byref(p)) == 0 and p.rr == pytest.approx(0.25)
    bad = C.c_void_p()
    assert lib.krr_wf_create_json(b"{", C.byref(bad)) == 1 and not bad.value
