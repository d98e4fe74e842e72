"""The C-ABI library builds, loads and exports every declared symbol (CPU)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="session")
def built():
    from swift_gb300 import build as b
    return b.build()


def declared_functions():
    src = open(os.path.join(ROOT, "include", "swift_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(swift_[a-z_0-9]+)\s*\(", src)))


def test_header_declares_functions():
    names = declared_functions()
    assert "swift_align" in names and "swift_sw_batch" in names and len(names) >= 17


def test_library_exports_every_declared_symbol(built):
    lib = C.CDLL(built)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_lists_match_header():
    import swift_gb300 as sg
    assert sorted(sg.EXPORTS) == declared_functions()


def test_params_defaults_match_reference(built):
    # src/common.h:29-75 and src/main.cu:52-62
    import swift_gb300 as sg
    p = sg.default_params()
    assert (p.seed_len, p.ignore_thres, p.max_hits) == (12, 1000, 3)
    assert (p.match, p.mismatch, p.gap_open, p.gap_ext) == (2, -1, -10, -1)
    assert p.qry_len == 0 and p.device_mem == 0


def test_no_device_is_an_error_not_a_crash(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    import swift_gb300 as sg
    with pytest.raises(sg.SwiftError):
        sg.Context(0)


def test_cli_usage_without_arguments(built):
    import subprocess
    import swift_gb300 as sg
    if not os.path.exists(sg.CLI_PATH):
        pytest.skip("CLI not built")
    r = subprocess.run([sg.CLI_PATH], capture_output=True, text=True)
    assert r.returncode == 0 and "USAGE" in r.stdout and "-q     Query fasta file" in r.stdout
    r = subprocess.run([sg.CLI_PATH, "-v"], capture_output=True, text=True)
    assert r.stdout.strip() == "Version: 0.11.2"
