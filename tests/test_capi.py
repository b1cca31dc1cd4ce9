"""CPU tests of the C ABI: the library loads, exports every declared symbol,
and its host-side logic (sizes, configs, argument checks) works without a GPU."""
import ctypes
import os
import re

import pytest

from althea_gb300 import ibl

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            text = open(os.path.join(ROOT, "include", f)).read()
            names |= set(re.findall(r"\b(althea_(?:ibl|ssr)_[a-z0-9_]+)\s*\(", text))
            names |= set(re.findall(r"\b(althea_ssr_convolve)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    L = ibl.load()
    syms = declared_symbols()
    assert len(syms) >= 19
    for s in syms:
        assert hasattr(L, s), s


def test_chain_geometry():
    assert ibl.chain_levels(4096, 2048) == 13
    assert ibl.chain_texels(4096, 2048) == sum(max(4096 >> l, 1) * max(2048 >> l, 1)
                                               for l in range(13))
    assert ibl.chain_level_offset(4096, 2048, 1) == 4096 * 2048
    assert ibl.chain_levels(37, 19) == 6
    assert ibl.load().althea_ibl_abi_version() == 2


def test_reference_config_matches_reference_bake():
    c = ibl.reference_config(4096, 2048)
    # Src/ImageBasedLighting.cpp:184-221 and PreFilterEnvMap.comp:5
    assert (c.irradiance_width, c.irradiance_height) == (4096, 2048)
    assert c.mip_count == 5 and (c.first_mip_width, c.first_mip_height) == (2048, 1024)
    assert c.samples == 10000 and c.generator == ibl.GEN_REF_HASH


def test_irradiance_workspace_sizes():
    L = ibl.load()
    assert L.althea_ibl_irradiance_workspace_size(4096, 2048, 128, 64) > 0
    # 300 x int(300*H/W) grid: W > 300 H gives no phi steps -> unsupported
    assert L.althea_ibl_irradiance_workspace_size(1000, 1, 8, 8) == 0


def test_argument_checks_without_gpu():
    L = ibl.load()
    assert L.althea_ibl_build_env_chain(None, 4, 4, None, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_build_env_chain(16, 0, 4, 16, None) == ibl.ERR_INVALID_ARGUMENT
    assert b"env size" in L.althea_ibl_last_error()
    assert L.althea_ibl_prefilter(None, 8, 8, None, 0, 16, 0, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_brdf_lut(None, 8, 64, 16, 0, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_brdf_lut(16, 8, 64, 16, 7, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_irradiance(16, 1000, 1, 16, 8, 8, 128, 16, 1 << 20, None) == \
        ibl.ERR_UNSUPPORTED
    assert L.althea_ibl_irradiance_noalloc(16, 64, 32, None, 8, 8, 128, None) == \
        ibl.ERR_INVALID_ARGUMENT
    bad = ibl.Config()
    ctx = ctypes.c_void_p()
    assert L.althea_ibl_create(ctypes.byref(bad), ctypes.byref(ctx)) == ibl.ERR_INVALID_ARGUMENT
    assert not ctx.value
    # config checks come before any device work, so they answer without a GPU
    for field, value, what in (("mip_count", 0, b"mip_count"), ("samples", 0, b"samples"),
                               ("lut_orientation", 7, b"lut_orientation"),
                               ("lut_samples", 0, b"lut_samples"),
                               ("irradiance_width", 100000, b"irradiance size")):
        cfg = ibl.make_config(64, 32, lut_size=16)
        setattr(cfg, field, value)
        assert L.althea_ibl_create(ctypes.byref(cfg), ctypes.byref(ctx)) == \
            ibl.ERR_INVALID_ARGUMENT, field
        assert what in L.althea_ibl_last_error() and not ctx.value
    assert L.althea_ibl_bake(None, None, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_bake_status(None, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_context_device_bytes(None) == 0
    n = ctypes.c_int(7)
    assert L.althea_ibl_contraction_times(None, None, 0, ctypes.byref(n)) == \
        ibl.ERR_INVALID_ARGUMENT


def test_context_path_and_format_checks_without_gpu():
    """The bake context's path and output format: values outside the enums
    are invalid, RGBA16F is refused on the plain path, and a precision config
    the planner cannot run is refused at create -- all before any device work."""
    L = ibl.load()
    ctx = ctypes.c_void_p()
    ref = ibl.reference_config(4096, 2048)
    assert (ref.path, ref.out_format) == (ibl.PATH_PLAIN, ibl.FORMAT_RGBA32F)
    for field, value, status, what in (
            ("path", 2, ibl.ERR_INVALID_ARGUMENT, b"path 2"),
            ("out_format", 5, ibl.ERR_INVALID_ARGUMENT, b"out_format 5"),
            ("out_format", ibl.FORMAT_RGBA16F, ibl.ERR_UNSUPPORTED, b"plain path")):
        cfg = ibl.make_config(64, 32)
        setattr(cfg, field, value)
        assert L.althea_ibl_create(ctypes.byref(cfg), ctypes.byref(ctx)) == status, field
        assert what in L.althea_ibl_last_error() and not ctx.value
    # irradiance 100 wide does not divide its 2048-wide source level
    cfg = ibl.make_config(4096, 2048, irradiance_size=(100, 50), mip_count=9,
                          path=ibl.PATH_PRECISION, out_format=ibl.FORMAT_RGBA16F)
    assert L.althea_ibl_create(ctypes.byref(cfg), ctypes.byref(ctx)) == ibl.ERR_UNSUPPORTED
    assert b"precision path" in L.althea_ibl_last_error() and not ctx.value


def test_noalloc_size_limit_without_gpu():
    """The no-allocation irradiance holds 4 MiB of partial sums: 512 x 512
    output texels (one 16-byte partial each) fit exactly, one texel more is
    refused before any device work."""
    L = ibl.load()
    assert L.althea_ibl_irradiance_workspace_size(1024, 512, 512, 512) == 4 * 1024 * 1024
    assert L.althea_ibl_irradiance_workspace_size(1024, 512, 545, 481) > 4 * 1024 * 1024
    fake = 1 << 20  # aligned, never dereferenced: the size check answers first
    assert L.althea_ibl_irradiance_noalloc(fake, 1024, 512, fake, 545, 481, 545 * 16, None) == \
        ibl.ERR_UNSUPPORTED
    assert b"no-allocation" in L.althea_ibl_last_error()


def test_python_errors_carry_status():
    with pytest.raises(ibl.IBLError) as e:
        ibl._check(ibl.ERR_UNSUPPORTED)
    assert e.value.status == ibl.ERR_UNSUPPORTED


def test_wait_selftest_rejects_bad_limits_without_gpu():
    L = ibl.load()
    assert L.althea_ibl_tc_wait_selftest(0, None, None) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_tc_wait_selftest(2 * 10**9, None, None) == ibl.ERR_INVALID_ARGUMENT


def test_precision_planner_levels_without_gpu():
    """The source level per output (host logic only): W/4-wide sources for
    roughness <= 0.40, W/2 for rougher mips and the irradiance, never coarser
    than the output, -1 for roughness 0."""
    mips = [(2048 >> m, 1024 >> m) for m in range(9)]
    rough = [m / 8 for m in range(9)]
    levels, irr = ibl.tc_plan(4096, 2048, mips, rough, 128)
    assert levels == [-1, 2, 2, 2, 1, 1, 1, 1, 1] and irr == 1
    spec = ibl.spec_for(2048, 1024)
    levels, irr = ibl.tc_plan(2048, 1024, spec.mip_sizes, spec.roughness, 32)
    assert levels == [-1, 1, 1, 0, 0, 0, 0, 0] and irr == 0
    for w in (256, 512, 1024):
        spec = ibl.spec_for(w, w // 2)
        levels, irr = ibl.tc_plan(w, w // 2, spec.mip_sizes, spec.roughness, 32)
        assert levels[0] == -1 and all(l == 0 for l in levels[1:]) and irr == 0


def test_precision_workspace_sizes_without_gpu():
    L = ibl.load()
    arr = (ibl.MipTarget * 2)(ibl.MipTarget(0, 16 * 256, 256, 128, 0.3),
                              ibl.MipTarget(0, 16 * 8, 8, 4, 1.0))
    assert L.althea_ibl_tc_workspace_size(1024, 512, arr, 2, None, 32, 16, -1) > 0
    # an output width that does not divide the source level's width: unsupported
    bad = (ibl.MipTarget * 1)(ibl.MipTarget(0, 16 * 96, 96, 48, 0.3))
    assert L.althea_ibl_tc_workspace_size(4096, 2048, bad, 1, None, 0, 0, -1) == 0


def test_precision_source_levels_must_exist_in_the_chain():
    """A caller-named source level past the chain's last level is refused
    before any pointer into the chain is formed."""
    L = ibl.load()
    w, h = 64, 32  # levels 0..6
    one = (ibl.MipTarget * 1)(ibl.MipTarget(0, 16, 1, 1, 0.5))
    assert L.althea_ibl_tc_workspace_size(w, h, one, 1, (ctypes.c_int * 1)(6), 0, 0, -1) > 0
    assert L.althea_ibl_tc_workspace_size(w, h, one, 1, (ctypes.c_int * 1)(7), 0, 0, -1) == 0
    assert b"source level 7" in L.althea_ibl_last_error()
    assert L.althea_ibl_tc_workspace_size(w, h, one, 1, (ctypes.c_int * 1)(40), 0, 0, -1) == 0
    assert L.althea_ibl_tc_workspace_size(w, h, None, 0, None, 1, 1, 7) == 0
    assert b"irradiance source level 7" in L.althea_ibl_last_error()
    # contracted outputs are at most 1024 wide; roughness 0 (the delta path) is not contracted
    for mw, r, ok in ((1024, 0.5, True), (2048, 0.5, False), (2048, 0.0, True)):
        t = (ibl.MipTarget * 1)(ibl.MipTarget(0, 16 * mw, mw, mw // 2, r))
        assert (L.althea_ibl_tc_workspace_size(4096, 2048, t, 1, None, 0, 0, -1) > 0) == ok
    assert L.althea_ibl_tc_workspace_size(4096, 2048, None, 0, None, 2048, 1024, -1) == 0
    # counts outside 0..MAX_MIPS, or mips missing, are refused without touching them
    assert L.althea_ibl_tc_workspace_size(w, h, None, 2, None, 0, 0, -1) == 0
    assert L.althea_ibl_tc_workspace_size(w, h, one, ibl.MAX_MIPS + 1, None, 0, 0, -1) == 0
    lv, il = (ctypes.c_int * 1)(), ctypes.c_int()
    assert L.althea_ibl_tc_plan(w, h, None, 1, 0, lv, ctypes.byref(il)) == ibl.ERR_INVALID_ARGUMENT
    assert L.althea_ibl_tc_plan(w, h, one, -1, 0, lv, ctypes.byref(il)) == ibl.ERR_INVALID_ARGUMENT
    # the planner's own choices always name existing levels
    for ew in (16, 256, 4096):
        for mw in (1, 2, ew // 2):
            lv1 = (ctypes.c_int * 1)()
            t = (ibl.MipTarget * 1)(ibl.MipTarget(0, 16 * mw, mw, max(mw // 2, 1), 0.7))
            assert L.althea_ibl_tc_plan(ew, ew // 2, t, 1, mw, lv1, ctypes.byref(il)) == ibl.OK
            assert 0 <= lv1[0] < ibl.chain_levels(ew, ew // 2)
            assert 0 <= il.value < ibl.chain_levels(ew, ew // 2)


# ctypes mirror -> C type of include/althea_ibl.h
_LAYOUTS = [
    (ibl.MipTarget, "althea_ibl_mip_target"), (ibl.Config, "althea_ibl_config"),
    (ibl.Outputs, "althea_ibl_outputs"), (ibl.Probe, "althea_ibl_probe"),
    (ibl.BatchParams, "althea_ibl_batch_params"), (ibl.BatchInfo, "althea_ibl_batch_info"),
    (ibl.ServerConfig, "althea_ibl_server_config"), (ibl.Request, "althea_ibl_request"),
    (ibl.Completion, "althea_ibl_completion"), (ibl.ServerStats, "althea_ibl_server_stats"),
    (ibl.Sun, "althea_ibl_sun"), (ibl.TcWork, "althea_ibl_tc_work"),
]
# Python constant -> C enum constant or macro
_CONSTANTS = {
    "OK": "ALTHEA_IBL_OK", "ERR_INVALID_ARGUMENT": "ALTHEA_IBL_ERR_INVALID_ARGUMENT",
    "ERR_CUDA": "ALTHEA_IBL_ERR_CUDA", "ERR_OUT_OF_MEMORY": "ALTHEA_IBL_ERR_OUT_OF_MEMORY",
    "ERR_UNSUPPORTED": "ALTHEA_IBL_ERR_UNSUPPORTED", "ERR_BUDGET": "ALTHEA_IBL_ERR_BUDGET",
    "ERR_NOT_READY": "ALTHEA_IBL_ERR_NOT_READY", "GEN_REF_HASH": "ALTHEA_IBL_GEN_REF_HASH",
    "GEN_HAMMERSLEY": "ALTHEA_IBL_GEN_HAMMERSLEY", "LUT_ASSET": "ALTHEA_IBL_LUT_ASSET",
    "LUT_CORRECTED": "ALTHEA_IBL_LUT_CORRECTED", "MAX_MIPS": "ALTHEA_IBL_MAX_MIPS",
    "BATCH_AUTOTUNE": "ALTHEA_IBL_BATCH_AUTOTUNE", "BATCH_GRAPH": "ALTHEA_IBL_BATCH_GRAPH",
    "BATCH_PRECISION": "ALTHEA_IBL_BATCH_PRECISION", "BATCH_HALF": "ALTHEA_IBL_BATCH_HALF",
    "PATH_PLAIN": "ALTHEA_IBL_PATH_PLAIN", "PATH_PRECISION": "ALTHEA_IBL_PATH_PRECISION",
    "FORMAT_RGBA32F": "ALTHEA_IBL_FORMAT_RGBA32F", "FORMAT_RGBA16F": "ALTHEA_IBL_FORMAT_RGBA16F",
    "MAX_SUNS": "ALTHEA_IBL_MAX_SUNS",
}


def test_ctypes_mirror_matches_the_header(tmp_path):
    """Every ctypes structure of the Python binding has the size and field
    offsets the C compiler gives the header's struct, and every mirrored
    constant has the header's value (gcc on a generated probe program)."""
    import shutil
    import subprocess
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "althea_ibl.h"',
             "int main(void) {"]
    for cls, ctype in _LAYOUTS:
        lines.append(f'  printf("{ctype} size %zu\\n", sizeof({ctype}));')
        for name, _ in cls._fields_:
            lines.append(f'  printf("{ctype} {name} %zu\\n", offsetof({ctype}, {name}));')
    for py, c in _CONSTANTS.items():
        lines.append(f'  printf("const {py} %ld\\n", (long){c});')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-Wall", "-Werror", "-I",
                           os.path.join(ROOT, "include"), "-o", str(exe), str(src)])
    got = {}
    for line in subprocess.check_output([str(exe)], text=True).splitlines():
        a, b, v = line.split()
        got[(a, b)] = int(v)
    for cls, ctype in _LAYOUTS:
        assert got[(ctype, "size")] == ctypes.sizeof(cls), ctype
        for name, _ in cls._fields_:
            assert got[(ctype, name)] == getattr(cls, name).offset, (ctype, name)
    for py, c in _CONSTANTS.items():
        assert got[("const", py)] == getattr(ibl, py), (py, c)


def test_header_compiles_as_cpp(tmp_path):
    """The header is usable from the reference's C++ (extern "C", no C-only syntax)."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "use.cpp"
    src.write_text('#include "althea_ibl.h"\n'
                   'int f() { althea_ibl_config c; althea_ibl_config_reference(&c, 64, 32);\n'
                   '          return c.mip_count + althea_ibl_abi_version(); }\n')
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                           "-I", os.path.join(ROOT, "include"), str(src)])


def test_cpp_consumer_links_and_runs(tmp_path):
    """A C++ program (tests/capi_consumer.cpp) links the library through the
    header alone and runs its device-free calls: planner, configs, RGBE files,
    error reporting."""
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    lib = ibl.load()._name
    exe = tmp_path / "consumer"
    libdir = os.path.dirname(lib)
    cudart = "/usr/local/cuda/lib64"
    subprocess.check_call(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-O1",
                           "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "capi_consumer.cpp"), "-o", str(exe),
                           "-L", libdir, "-lalthea_ibl", "-Wl,-rpath," + libdir,
                           "-Wl,-rpath-link," + cudart, "-Wl,-rpath," + cudart])
    out = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=60)
    assert out.returncode == 0, out.stderr
    assert "consumer ok" in out.stdout
