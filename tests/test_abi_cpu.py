"""C-ABI shape checks that need no GPU: the library loads, exports every
symbol declared in include/*.h, and rejects bad arguments with AB_ERR_ARG
before touching the device."""
import glob
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(ab_\w+)\s*\(", src, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ("ab_unpack_4bit", "ab_unpack_1bit", "ab_ipfb", "ab_pfb", "ab_avg_xcorr_all_ant",
                 "ab_xcorr_coarse_4bit", "ab_stream_create", "ab_stream_push"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"
    # every binding the Python layer uses is declared in the header
    assert set(_lib.SIGNATURES) <= set(declared_symbols())


def test_integration_guide_binds_every_symbol():
    """Every declared entry point appears in the maintainer's binding guide."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    missing = [n for n in declared_symbols() if not re.search(rf"\b{n}\b", text)]
    assert not missing, f"no binding shown for: {missing}"


def test_bad_arguments_are_rejected_on_host():
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    assert lib.ab_unpack_4bit(None, None, None, 0, 10, None, 4, 8, None) == -1
    assert b"NULL" in lib.ab_last_error()
    assert lib.ab_sortpols(1, 1, 1, 0, 1, 1, 8, 3, 0, 8, None) == -1
    assert lib.ab_strerror(-3) == b"unsupported size"
    assert lib.ab_version() >= 10000


def test_ops_fail_loudly_without_gpu():
    import torch
    if torch.cuda.is_available():
        pytest.skip("GPU present")
    import numpy as np
    from albatros_axion_detection_gb300 import unpacking
    with pytest.raises((RuntimeError, TypeError)):
        unpacking.unpack_4bit(np.zeros((4, 8), np.uint8), 0, 4, np.arange(4), 4)


def test_new_entry_points_check_arguments_on_host():
    """Histogram and ingest entry points reject bad arguments before any
    CUDA call (so this runs without a GPU)."""
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    call = lambda name, *a: getattr(lib, name)(*a)
    assert call("ab_hist", None, None, 0, 4, 8, 4, 0, None) == -1                      # NULL data
    assert call("ab_hist", 16, 16, 0, 4, 8, 2, 0, None) == -1                          # bit depth 2
    assert call("ab_hist", 16, 16, 0, 4, 8, 4, 3, None) == -1                          # mode 3
    assert call("ab_hist", 16, 16, 0, 4, 7, 1, 0, None) == -1                          # odd 1-bit channels
    assert call("ab_hist", 17, 16, 0, 4, 8, 4, 0, None) == -1                          # odd 4-bit address
    assert call("ab_packets_to_rows", None, 4, 24, 16, None) == -1
    assert call("ab_packets_to_rows", 16, 4, 4, 16, None) == -1                        # no payload
    assert call("ab_spec_map_add", 16, 4, 0, 0, 0, 16, 8, None) == -1                  # spp 0
    assert call("ab_spec_map_add", 16, 4, 5, (1 << 31) - 4, 0, 16, 8, None) == -1      # rows beyond int32
    assert call("ab_spec_map_init", None, 8, None) == -1
    assert call("ab_spec_map_finish", None, 8, None) == -1
    assert b"ab_" in lib.ab_last_error()


def test_every_entry_point_rejects_bad_arguments_on_host():
    """Each compute entry point returns AB_ERR_ARG (-1) for NULL pointers or
    impossible sizes before any CUDA call, so these run without a GPU; NULL
    objects are harmless to destroy and read back as -1 / NULL."""
    import ctypes
    from albatros_axion_detection_gb300 import _lib
    lib = _lib.load()
    bad = [
        ("ab_unpack_1bit", None, None, None, 0, 10, None, 4, 8, None),
        ("ab_unpack_1bit", 16, 16, 16, 0, 10, 16, 4, 7, None),               # odd 1-bit channel count
        ("ab_unpack_4bit_i8", None, None, None, 0, 10, None, 4, 8, None),
        ("ab_unpack_1bit_i8", 16, 16, 16, 0, 10, 16, 4, 7, None),
        ("ab_unpack_4bit_range", 16, 16, 16, 0, 10, 1, 4, 8, None),          # range not 4-aligned
        ("ab_unpack_4bit", 16, 16, 16, 5, 2, 16, 4, 8, None),                # rowend < rowstart
        ("ab_make_continuous", 16, 4, 2, 16, 0, 16, 0, 8, 16, None),         # nspec 0
        ("ab_calculate_filter", None, None, 10, 0.45, None),
        ("ab_get_matft", None, 16, 64, 2049, 4, None),
        ("ab_build_filter", None, 16, 64, 2049, 4, 0.45, None),
        ("ab_ipfb", None, 16, 16, 16, 64, 2049, None),
        ("ab_pfb", None, 16, 4096 * 8, 16, 2049, 4, 16, None),
        ("ab_pfb_band", None, 16, 4096 * 8, 16, 2049, 4, 0, 64, 16, None),
        ("ab_avg_xcorr_all_ant", None, 2, 2, 10, 4, 16, None),
        ("ab_avg_xcorr_all_ant", 16, 0, 2, 10, 4, 16, None),                 # no antennas
        ("ab_xcorr_coarse_4bit", None, 16, 100, 2, 100, 8, 0, 10, None, 16, 4, 0, 16, 16, None),
        ("ab_xcorr_coarse_4bit_noalloc", 16, 100, 2, 100, 8, 90, 20, None, 16, 4, 0, 16, 16, None),  # rows past nspec
        ("ab_xcorr_coarse_4bit_noalloc", 16, 100, 40, 100, 8, 0, 20, None, 16, 4, 0, 16, 16, None),  # 40 antennas
        # channel or chunk counts whose scratch size would wrap a 64-bit product
        ("ab_xcorr_coarse_4bit_noalloc", 16, 1 << 50, 32, 1 << 40, 8, 0, 1 << 40, None, 16, 1 << 40, 1, 16, 16,
         None),
        ("ab_xcorr_coarse_4bit_noalloc", 16, 1 << 50, 32, 1 << 40, 8, 0, 1 << 40, None, 16, 1 << 20, 1, 16, 16,
         None),
        ("ab_avg_xcorr_4bit_pairs", None, 16, 16, 16, 4, 4, 16, 16, None),
        ("ab_avg_xcorr_1bit_pairs", None, 16, 16, 16, 4, 4, 8, 16, None),
        ("ab_stream_create", None, 2, 64, 4, 16, 16, 64, 32768, 80, 64, 4, 0.45, 512, 2, 0, 4096,
         ctypes.byref(ctypes.c_void_p())),
        ("ab_stream_push", None, 16, 100, None, 0, 0, None),
        ("ab_stream_push_final", None, 16, 100, None, 0, 0, None),
        ("ab_stream_reset", None, None),
        ("ab_stream_profile", None, 1),
        ("ab_stream_stage_times", None, 16, 16),
        ("ab_stream_time_filter", None, 16, 16),
        ("ab_stream_set_workspace", None, 16, 100),
        ("ab_ctx_set_option", None, 3, 8),
        ("ab_ctx_set_time_filter", None, 0, 16),
        ("ab_ctx_set_fft_plan", None, 16, None, 0),
    ]
    for name, *args in bad:
        assert getattr(lib, name)(*args) == -1, (name, args, lib.ab_last_error())
        assert lib.ab_last_error().startswith(name.encode()[:9]), (name, lib.ab_last_error())
    for name in ("ab_stream_kernel_launches", "ab_stream_fir_taps", "ab_stream_workspace_bytes"):
        assert getattr(lib, name)(None) == -1
    assert lib.ab_stream_vis(None) is None
    assert lib.ab_stream_destroy(None) == 0 and lib.ab_ctx_destroy(None) == 0


def test_integration_guide_argtypes_match_the_bindings():
    """The argtypes lists shown in the binding guide agree with the
    package's own ctypes signatures (same count, same C type sizes)."""
    import ctypes
    from albatros_axion_detection_gb300 import _lib
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    env = {"P": ctypes.c_void_p, "I64": ctypes.c_int64, "D": ctypes.c_double, "ctypes": ctypes}
    shown = re.findall(r"^ab\.(ab_\w+)\.argtypes = (\[.*?\])", text, flags=re.M)
    assert len(shown) >= 30
    for name, lst in shown:
        doc = eval(lst, env)
        if name not in _lib.SIGNATURES:
            continue  # ab_ctx_create takes an out-pointer; bound separately in _lib
        ours = _lib.SIGNATURES[name][1]
        assert len(doc) == len(ours), name
        kind = lambda t: ("f" if t in (ctypes.c_double, ctypes.c_float) else "i", ctypes.sizeof(t))
        for a, b in zip(doc, ours):  # doubles travel in other registers than integers and pointers
            assert kind(a) == kind(b), (name, a, b)


def test_python_signatures_match_the_header():
    """Every ctypes signature the package binds has the header's argument
    count and C types (pointer, 32/64-bit integer, double), return included."""
    import ctypes
    from albatros_axion_detection_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "albatros_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    protos = {m.group(2): (m.group(1), m.group(3))
              for m in re.finditer(r"^\s*((?:const\s+)?[\w ]+?\s*\**)\s*(ab_\w+)\s*\(([^)]*)\)\s*;", src, flags=re.M)}

    def ckind(decl):
        decl = decl.strip()
        if "*" in decl:
            return ("i", 8)
        if decl.startswith("double"):
            return ("f", 8)
        if decl.startswith("int64_t"):
            return ("i", 8)
        if decl.startswith(("int32_t", "int")):
            return ("i", 4)
        raise AssertionError(decl)

    def pkind(t):
        return ("f" if t in (ctypes.c_double, ctypes.c_float) else "i", ctypes.sizeof(t))

    for name, (res, args) in _lib.SIGNATURES.items():
        ret, params = protos[name]
        params = [] if params.strip() in ("", "void") else params.split(",")
        assert len(params) == len(args), name
        for decl, t in zip(params, args):
            assert ckind(decl) == pkind(t), (name, decl, t)
        assert ckind(ret) == pkind(res), (name, ret, res)
