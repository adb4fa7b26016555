"""C-ABI checks that need no GPU: the library builds and loads, exports every entry point
declared in include/stormbird_gb300.h, and rejects bad setups with the documented codes
before any CUDA call (the reference returns a serde error here: simulation_builder.rs:81-88)."""
import ctypes
import json
import os
import re

import pytest

from stormbird_gb300 import setups as S
from stormbird_gb300._abi import StepOutput

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "stormbird_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(gpu_lib, n), f"{n} declared in the header but not exported"


def test_python_signatures_cover_header():
    from stormbird_gb300.native import SIGNATURES

    assert sorted(n for n, _, _ in SIGNATURES) == declared_functions()


def test_step_output_struct_layout():
    # 10 pointers, 2 x double[3], residual, int64, 2 x int32
    assert ctypes.sizeof(StepOutput) == 10 * 8 + 6 * 8 + 8 + 8 + 8


def _new(gpu_lib, js: str):
    h = gpu_lib.sb_sim_new(js.encode(), 0)
    return h, gpu_lib.sb_last_status(), gpu_lib.sb_last_error().decode()


@pytest.mark.parametrize("doc,code,fragment", [
    ("{not json", -3, "JSON parse error"),
    ("{}", -3, "missing field `line_force_model`"),
    (json.dumps({"line_force_model": {"wing_builders": [], "nr_sections": 4}}), -3, "at least one wing"),
])
def test_bad_setup_is_rejected(gpu_lib, doc, code, fragment):
    h, st, msg = _new(gpu_lib, doc)
    assert not h and st == code and fragment in msg


def test_unknown_field_is_rejected(gpu_lib):
    d = json.loads(S.wing_sail_row(1, 4, 5))
    d["simulation_settings"]["Dynamic"]["wake"]["not_a_field"] = 1
    h, st, msg = _new(gpu_lib, json.dumps(d))
    assert not h and st == -3 and "unknown field `not_a_field`" in msg


def test_unsupported_section_model(gpu_lib):
    d = json.loads(S.wing_sail_row(1, 4, 5))
    d["line_force_model"]["wing_builders"][0]["section_model"] = {"RotatingCylinder": {}}
    h, st, msg = _new(gpu_lib, json.dumps(d))
    assert not h and st == -7 and "RotatingCylinder" in msg


def test_null_arguments(gpu_lib):
    assert not gpu_lib.sb_sim_new(None, 0)
    assert gpu_lib.sb_last_status() == -1
    assert gpu_lib.sb_sim_sizes(None, None, None, None) == -1
    gpu_lib.sb_sim_free(None)  # accepted


def test_oracle_accepts_reference_python_builder_json(oracle_mod):
    """The setup JSON the reference's own Python builders emit (interfaces/stormbird_setup)
    is read with Rust defaults (committed fixture from tests/golden/make_golden.py)."""
    path = os.path.join(ROOT, "tests", "golden", "setup_stormbird_setup_dynamic.json")
    js = open(path).read()
    sim = oracle_mod.OracleSimulation(js)
    assert sim.nr_span_lines == 2 * 16
