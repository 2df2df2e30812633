"""CPU tests of the C-ABI boundary: the library builds, loads and exports every symbol that
include/dic.h declares; the ctypes structs match the C layouts; without a GPU the engine
fails loudly instead of falling back to anything."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "dic.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dic_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libpath():
    from fasticgn_gb300 import _build
    return _build.build_lib()


def test_header_declarations_are_bound(libpath):
    from fasticgn_gb300 import _lib
    names = declared_functions()
    assert len(names) >= 18
    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_library_exports_every_declared_symbol(libpath):
    out = subprocess.run(["nm", "-D", "--defined-only", str(libpath)], capture_output=True, text=True,
                         check=True).stdout
    exported = set(re.findall(r"\bT (dic_[a-z_0-9]+)", out))
    missing = set(declared_functions()) - exported
    assert not missing, missing
    lib = ctypes.CDLL(str(libpath))
    for name in declared_functions():
        assert hasattr(lib, name)


def test_struct_layouts_match_header(tmp_path):
    from fasticgn_gb300 import _lib
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include <stddef.h>\n#include "dic.h"\n'
                   'int main(void){printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(dic_poi),'
                   ' sizeof(dic_config), sizeof(dic_stats), sizeof(dic_frame_policy), sizeof(dic_frame_report),'
                   ' offsetof(dic_poi, zncc), offsetof(dic_stats, icgn_iterations), sizeof(dic_job),'
                   ' offsetof(dic_job, pois), sizeof(dic_batch_report), sizeof(dic_launch_shape),'
                   ' offsetof(dic_launch_shape, tile), sizeof(dic_tuning)); return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
    got = list(map(int, subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()))
    want = [_lib.POI_DTYPE.itemsize, ctypes.sizeof(_lib.DicConfig), ctypes.sizeof(_lib.DicStats),
            ctypes.sizeof(_lib.DicFramePolicy), ctypes.sizeof(_lib.DicFrameReport),
            _lib.POI_DTYPE.fields["zncc"][1], _lib.DicStats.icgn_iterations.offset, ctypes.sizeof(_lib.DicJob),
            _lib.DicJob.pois.offset, ctypes.sizeof(_lib.DicBatchReport), ctypes.sizeof(_lib.DicLaunchShape),
            _lib.DicLaunchShape.tile.offset, ctypes.sizeof(_lib.DicTuning)]
    assert got == want


def test_version_and_abi(libpath):
    from fasticgn_gb300 import _lib
    L = _lib.load()
    assert L.dic_abi_version() == 2
    assert b"sm_103a" in L.dic_version()


def test_null_arguments_are_rejected(libpath):
    from fasticgn_gb300 import _lib
    L = _lib.load()
    assert L.dic_engine_create(None, None) == _lib.DIC_ERR_ARGUMENT
    assert L.dic_icgn(None, None, 0) == _lib.DIC_ERR_ARGUMENT
    L.dic_engine_destroy(None)
    assert L.dic_last_error(None) == b"null engine"


def test_engine_without_gpu_fails_loudly(libpath):
    torch = pytest.importorskip("torch")
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from fasticgn_gb300 import Engine, DicError
    with pytest.raises(DicError):
        Engine(15)


def test_grid_queue_matches_build_poi_queue():
    """buildPoiQueue (opencorr_cli_cuda_mvp.cpp:2439-2472): margin r+2, y outer, x inner."""
    from fasticgn_gb300 import grid_queue
    q = grid_queue(64, 48, 7, 5)
    xs = list(range(9, 64 - 9, 5))
    ys = list(range(9, 48 - 9, 5))
    assert len(q) == len(xs) * len(ys)
    assert q["x"][0] == 9 and q["y"][0] == 9
    assert list(q["x"][:len(xs)]) == xs
    assert list(q["y"][::len(xs)]) == ys
    ql = grid_queue(64, 48, 7, 5, lines=[20, 3, 20])
    assert len(ql) == 2 * len(xs) and list(ql["y"][::len(xs)]) == [20, 20]
