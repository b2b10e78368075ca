"""CPU tests of the C-ABI boundary: the library builds, loads and exports every
symbol of include/abcgpu.h, the ctypes mirror matches the C struct layout, and
argument validation fails cleanly (no kernel is launched here)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from abc_inference_transcription_gb300 import abi
from abc_inference_transcription_gb300.config import make_config
from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "abcgpu.h")


def declared_symbols():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^\s*(?:int|void\*|const char\*)\s+(abc_\w+)\(", src, re.M)))


def test_header_declares_the_abi_list():
    assert declared_symbols() == sorted(abi.ABI_SYMBOLS)


def test_library_exports_every_declared_symbol(built):
    lib = abi.load_library()
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", abi.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (abc_\w+)", out))
    assert set(declared_symbols()) <= exported


def test_struct_layout_matches_c(tmp_path):
    prog = tmp_path / "layout.c"
    prog.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "abcgpu.h"\n'
        "int main(void){printf(\"%zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(abc_config), offsetof(abc_config, ages),"
        " offsetof(abc_config, pulse_stat_cond), offsetof(abc_config, event_cap), sizeof(abc_prior),"
        " offsetof(abc_prior, vary_mode), offsetof(abc_prior, factor));return 0;}\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(prog), "-o", str(exe)], check=True)
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    want = [C.sizeof(abi.AbcConfig), abi.AbcConfig.ages.offset, abi.AbcConfig.pulse_stat_cond.offset,
            abi.AbcConfig.event_cap.offset, C.sizeof(abi.AbcPrior), abi.AbcPrior.vary_mode.offset,
            abi.AbcPrior.factor.offset]
    assert got == want


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def test_create_validates_before_touching_cuda(built):
    lib = abi.load_library()
    h = C.c_void_p()
    bad = make_config("hour")
    bad.ages[0] = 25.0  # outside (0, cycle)
    assert lib.abc_create(C.byref(h), C.byref(bad)) == abi.ERR_INVALID
    bad = make_config("hour")
    bad.n_steps = 0
    assert lib.abc_create(C.byref(h), C.byref(bad)) == abi.ERR_INVALID
    bad = make_config("hour")
    bad.pulse[10] = 200.0  # labelling would start before t0
    assert lib.abc_create(C.byref(h), C.byref(bad)) == abi.ERR_INVALID


def test_create_without_gpu_reports_cuda_error(built):
    if _has_gpu():
        pytest.skip("a GPU is visible")
    lib = abi.load_library()
    h = C.c_void_p()
    assert lib.abc_create(C.byref(h), C.byref(make_config("hour"))) == abi.ERR_CUDA
    assert lib.abc_destroy(None) == 0
    assert lib.abc_num_params(None, 1) == abi.ERR_INVALID


def test_num_params_mirror():
    cfg = make_config("hour")
    assert [abi.num_params(cfg, m) for m in range(1, 6)] == [5, 5, 9, 9, 9]
    cfg = make_config("min", splicing=True, scaling_column=True)
    assert [abi.num_params(cfg, m) for m in range(1, 6)] == [7, 7, 11, 11, 11]
    with pytest.raises(ValueError):
        abi.num_params(cfg, 6)


def test_product_path_has_no_oracle_dependency():
    """The product never imports, links or includes the oracle."""
    pkg = os.path.join(ROOT, "abc_inference_transcription_gb300")
    bad = re.compile(r"(^\s*(from|import)\s+oracle)|abcoracle|abc_oracle|orc_", re.M)
    for root, _, files in os.walk(pkg):
        for f in files:
            if f.endswith((".py", ".cu", ".cuh", ".h")):
                assert not bad.search(open(os.path.join(root, f)).read()), f


def test_breakpoint_grid_detection(built):
    """The integer breakpoint path of the production SSA applies when every
    time of the configuration is a multiple of a power-of-two quantum."""
    from abc_inference_transcription_gb300 import abi
    assert abi.breakpoint_grid(make_config("hour")) == 0.25       # pulses of 15 min in hours
    assert abi.breakpoint_grid(make_config("min")) == 1.0         # whole minutes
    cfg = make_config("hour")
    cfg.pulse[0] = 0.1                                            # not a dyadic multiple
    assert abi.breakpoint_grid(cfg) is None
    cfg = make_config("hour")
    cfg.cycle = 21.0                                              # age step 4.2 h
    assert abi.breakpoint_grid(cfg) is None
