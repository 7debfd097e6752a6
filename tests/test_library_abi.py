"""CPU checks of the C ABI: the library builds for sm_103a, loads, and
exports every entry point declared in include/voxurf_gb300.h; the ctypes
struct mirrors match the header.  No compute calls (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "voxurf_gb300.h")


def _declared():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(vx_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from voxurf_gb300 import build

    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    names = _declared()
    assert len(names) >= 30, names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_ctypes_bindings_cover_header():
    from voxurf_gb300 import _abi, _native

    bound = set(_native.exported_names()) | set(_abi.struct_names())
    missing = [n for n in _declared() if n not in bound]
    assert not missing, missing


def test_status_strings(lib):
    lib.vx_status_string.restype = ctypes.c_char_p
    assert lib.vx_status_string(0) == b"ok"
    assert lib.vx_status_string(2) == b"output capacity exceeded"
    assert lib.vx_version() == 1


def test_struct_sizes_match_c_layout():
    """Every field of the ctypes mirrors is at the offset a C compiler gives
    the header's structs (checked by compiling a probe with gcc)."""
    import subprocess
    import tempfile

    from voxurf_gb300 import _abi

    structs = {"vx_grid_geom": _abi.GridGeom, "vx_fine_march_args": _abi.FineMarchArgs,
               "vx_fine_compact_args": _abi.FineCompactArgs, "vx_fine_feature_cfg": _abi.FineFeatureCfg,
               "vx_fine_features_args": _abi.FineFeaturesArgs, "vx_fine_composite_args": _abi.FineCompositeArgs,
               "vx_fine_composite_bwd_args": _abi.FineCompositeBwdArgs,
               "vx_fine_backward_args": _abi.FineBackwardArgs, "vx_coarse_march_args": _abi.CoarseMarchArgs,
               "vx_coarse_feature_cfg": _abi.CoarseFeatureCfg, "vx_coarse_features_args": _abi.CoarseFeaturesArgs,
               "vx_coarse_composite_args": _abi.CoarseCompositeArgs,
               "vx_coarse_composite_bwd_args": _abi.CoarseCompositeBwdArgs,
               "vx_coarse_backward_args": _abi.CoarseBackwardArgs, "vx_scene_desc": _abi.SceneDesc,
               "vx_view_chunk": _abi.ViewChunk, "vx_mlp_tc_args": _abi.MlpTcArgs,
               "vx_bg_sample_args": _abi.BgSampleArgs, "vx_cast_job": _abi.CastJob,
               "vx_fine_composite_loss_args": _abi.FineCompositeLossArgs, "vx_mlp_pack_job": _abi.MlpPackJob,
               "vx_mlp_train_fwd_args": _abi.MlpTrainFwdArgs, "vx_mlp_train_bwd_args": _abi.MlpTrainBwdArgs,
               "vx_mlp_wgrad_args": _abi.MlpWgradArgs, "vx_mlp_reduce_job": _abi.MlpReduceJob,
               "vx_mlp_f32_rowgemm_args": _abi.MlpF32RowGemmArgs, "vx_mlp_f32_wgrad_args": _abi.MlpF32WgradArgs,
               "vx_mlp_sum_job": _abi.MlpSumJob, "vx_womask_fg_alpha_args": _abi.WomaskFgAlphaArgs,
               "vx_womask_bg_alpha_args": _abi.WomaskBgAlphaArgs,
               "vx_womask_bg_features_args": _abi.WomaskBgFeaturesArgs,
               "vx_womask_composite_args": _abi.WomaskCompositeArgs, "vx_tv_loss_args": _abi.TvLossArgs}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "voxurf_gb300.h"', "int main(void){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "probe.c")
        open(c, "w").write("\n".join(lines))
        exe = os.path.join(d, "probe")
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split("\n")
    got = dict(line.split() for line in out if line)
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_every_called_entry_point_has_a_signature():
    """ctypes would pass undeclared arguments as 32-bit ints (truncating
    pointers): every vx_* name the package or bench.py uses is declared."""
    import glob
    import re

    from voxurf_gb300 import _abi, _native

    lib = _native.load()
    _abi._declare()
    names = set()
    for f in glob.glob(os.path.join(ROOT, "voxurf_gb300", "*.py")) + [os.path.join(ROOT, "bench.py")]:
        names |= set(re.findall(r'["\'](vx_[a-z0-9_]+)["\']', open(f).read()))
    undeclared = [n for n in sorted(names) if hasattr(lib, n) and getattr(lib, n).argtypes is None]
    assert not undeclared, undeclared
