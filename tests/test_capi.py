"""CPU tests of the C ABI: the library builds and loads, exports every symbol
the headers declare, and rejects bad arguments before touching the GPU."""
import ctypes as C
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = []
    for h in ("mhdgpu.h", "mhdgpu_compat.h", "mhdgpu_fortran.h"):
        src = open(os.path.join(REPO, "include", h)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", src, flags=re.M):
            name = m.group(1)
            if name not in ("defined",) and not name.isupper():
                names.append(name)
    return sorted(set(names))


@pytest.fixture(scope="module")
def L():
    import mhdgpu
    if not os.path.exists(mhdgpu.LIB_PATH):
        import build
        build.build()
    return mhdgpu.lib()


def test_headers_declare_the_python_export_list():
    import mhdgpu
    assert set(_declared_functions()) == set(mhdgpu.EXPORTS)


def test_library_exports_every_declared_symbol(L):
    for name in _declared_functions():
        assert hasattr(L, name), name


def test_status_strings(L):
    assert L.mhdgpu_status_string(0) == b"ok"
    assert L.mhdgpu_status_string(1) == b"invalid argument"
    assert b"sm_103a" in L.mhdgpu_version()


def test_bad_arguments_are_rejected_without_a_gpu(L):
    import mhdgpu
    P = C.c_void_p
    fake = P(0x1000)
    # zero-size box
    assert L.mhdgpu_fluidx(fake, fake, fake, 0, 4, 4, fake, None, None) == mhdgpu.MHD_ERR_ARG
    assert b"bad box" in L.mhdgpu_last_error()
    # pencil longer than the kernels accept
    assert L.mhdgpu_fluidx(fake, fake, fake, 4096, 1, 1, fake, None, None) == mhdgpu.MHD_ERR_ARG
    # null pointers
    assert L.mhdgpu_fluidx(None, fake, fake, 8, 8, 8, fake, None, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_advectbyzx(fake, fake, 8, 8, 8, fake, None, None) == mhdgpu.MHD_ERR_ARG
    # transposes must be out of place
    assert L.mhdgpu_transpose12(fake, fake, fake, fake, 8, 8, 8, None) == mhdgpu.MHD_ERR_ARG
    assert b"out of place" in L.mhdgpu_last_error()
    # bad CFL mode
    assert L.mhdgpu_cfl(fake, fake, 8, 8, 8, 7, fake, fake, None) == mhdgpu.MHD_ERR_ARG
    # negative step count, bad cfl number
    assert L.mhdgpu_advance(fake, fake, 8, 8, 8, -1, 0.9, 0, 0.0, fake, None, fake, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_advance(fake, fake, 8, 8, 8, 1, 0.0, 0, 0.0, fake, None, fake, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_advance(fake, fake, 8, 8, 8, 1, 0.9, 0, 0.0, fake, None, fake, 5, None) == mhdgpu.MHD_ERR_ARG
    # the step's own checks run before the CFL pass and the clock tick: with a
    # valid-looking clock, a null state, a null workspace or a y/z axis above
    # the pencil limit are rejected without a launch (no GPU is touched here)
    assert L.mhdgpu_advance(None, fake, 8, 8, 8, 1, 0.9, 0, 0.0, fake, None, fake, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_advance(fake, None, 8, 8, 8, 1, 0.9, 0, 0.0, fake, None, fake, 1, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_advance(fake, fake, 8, 8, 8, 1, 0.9, 0, 0.0, fake, None, None, 0, None) == mhdgpu.MHD_ERR_ARG
    assert b"null" in L.mhdgpu_last_error()
    assert L.mhdgpu_advance(fake, fake, 8, 2000, 8, 1, 0.9, 0, 0.0, fake, None, fake, 1, None) == mhdgpu.MHD_ERR_ARG
    assert b"MHD_MAX_PENCIL" in L.mhdgpu_last_error()
    assert L.mhdgpu_advance(fake, fake, 0, 8, 8, 1, 0.9, 0, 0.0, fake, None, fake, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_step_fused(fake, fake, 8, 2000, 8, fake, fake, None, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_dt_update(fake, -1.0, 0.0, fake, fake, None) == mhdgpu.MHD_ERR_ARG


def test_partial_overlap_rejected(L):
    import mhdgpu
    base = 0x100000
    n5 = 5 * 8 * 8 * 8 * 4
    st = L.mhdgpu_fluidx(C.c_void_p(base + 4), C.c_void_p(base), C.c_void_p(base + 10 * n5), 8, 8, 8,
                         C.c_void_p(base), None, None)
    assert st == mhdgpu.MHD_ERR_ARG


def test_tile_and_math_settings_without_a_gpu(L):
    import mhdgpu
    c, w, p = C.c_int(), C.c_int(), C.c_int()
    assert L.mhdgpu_get_tile(0, 128, C.byref(c), C.byref(w), C.byref(p)) == 0
    assert c.value * w.value * 32 >= 128
    assert L.mhdgpu_set_tile(0, 128, 3, 1, 1) == mhdgpu.MHD_ERR_ARG      # not compiled
    assert L.mhdgpu_set_tile(0, 300, 4, 1, 1) == mhdgpu.MHD_ERR_ARG      # does not cover
    assert L.mhdgpu_set_tile(0, 64, 2, 1, 16) == mhdgpu.MHD_ERR_ARG      # 512 threads
    assert L.mhdgpu_set_tile(2, 64, 2, 1, 1) == mhdgpu.MHD_ERR_ARG       # not a pencil kernel
    assert L.mhdgpu_set_math(7) == -1
    assert L.mhdgpu_set_math(0) == 0
    assert L.mhdgpu_set_row_staging(mhdgpu.MHD_STAGING_TMA) == mhdgpu.MHD_STAGING_CPASYNC   # the default
    assert L.mhdgpu_set_row_staging(mhdgpu.MHD_STAGING_CPASYNC) == mhdgpu.MHD_STAGING_TMA
    assert L.mhdgpu_set_row_staging(5) == -1
    assert L.mhdgpu_autotune(0, 4, 4, 0) == mhdgpu.MHD_ERR_ARG


def test_settings_are_per_host_thread(L):
    """The arithmetic policy, the row staging and the tile table set on one
    thread leave every other thread's launches as they were."""
    import threading
    import mhdgpu
    seen = {}

    def other():
        seen["math_before"] = L.mhdgpu_set_math(mhdgpu.MHD_MATH_FAST)
        seen["staging_before"] = L.mhdgpu_set_row_staging(mhdgpu.MHD_STAGING_TMA)
        seen["set_tile"] = L.mhdgpu_set_tile(0, 96, 4, 1, 2)
        seen["tile_there"] = mhdgpu.get_tile("fluidx", 96)

    assert L.mhdgpu_set_math(mhdgpu.MHD_MATH_FP64P) == mhdgpu.MHD_MATH_FAITHFUL
    here = mhdgpu.get_tile("fluidx", 96)
    assert here != (4, 1, 2)
    th = threading.Thread(target=other)
    th.start()
    th.join()
    assert seen == {"math_before": mhdgpu.MHD_MATH_FAITHFUL, "staging_before": mhdgpu.MHD_STAGING_CPASYNC,
                    "set_tile": 0, "tile_there": (4, 1, 2)}
    assert mhdgpu.get_tile("fluidx", 96) == here          # only the other thread's table changed
    assert L.mhdgpu_set_math(mhdgpu.MHD_MATH_FAITHFUL) == mhdgpu.MHD_MATH_FP64P
    assert L.mhdgpu_set_row_staging(mhdgpu.MHD_STAGING_CPASYNC) == mhdgpu.MHD_STAGING_CPASYNC


def test_workspace_sizes(L):
    assert L.mhdgpu_step_workspace_bytes(32, 32, 32) == 40 * 32 ** 3
    assert L.mhdgpu_advectbyzx_scratch_bytes(16, 8, 4) == 8 * 16 * 8 * 4
    assert L.mhdgpu_step_workspace_bytes(0, 1, 1) == 0
    assert L.mhdgpu_step_fused_workspace_bytes(32, 16, 8) == 8 * 32 * 16 * 8


def test_path_choice_and_host_entries_without_a_gpu(L):
    """MHD_PATH_AUTO's rule and its workspace, and the host-buffer entries'
    argument checks, all answered on the host."""
    import mhdgpu
    fused, plain, auto = mhdgpu.MHD_PATH_FUSED, mhdgpu.MHD_PATH_PLAIN, mhdgpu.MHD_PATH_AUTO
    assert L.mhdgpu_resolve_path(48, 48, 48) == fused
    assert L.mhdgpu_resolve_path(512, 32, 48) == fused        # x pencils are always contiguous
    assert L.mhdgpu_resolve_path(128, 128, 128) == plain
    assert L.mhdgpu_resolve_path(64, 256, 64) == plain
    assert L.mhdgpu_resolve_path(32, 32, 49) == plain
    for dims in ((128, 128, 128), (32, 256, 16)):
        want = (L.mhdgpu_step_fused_workspace_bytes(*dims) if L.mhdgpu_resolve_path(*dims) == fused
                else L.mhdgpu_step_workspace_bytes(*dims))
        assert L.mhdgpu_path_workspace_bytes(*dims, auto) == want
    assert L.mhdgpu_path_workspace_bytes(8, 8, 8, 9) == 0
    P = C.c_void_p
    fake, t = P(0x1000), C.c_float(0.0)
    args = (0.7, 0, C.byref(t), 0.0, 1, None, None)
    assert L.mhdgpu_run_host(None, fake, 8, 8, 8, *args, fused) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_run_host(fake, fake, 8, 8, 8, *args, 9) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_run_host(fake, fake, 0, 8, 8, *args, fused) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_release_host_cache() == mhdgpu.MHD_OK   # nothing cached: a no-op
    assert L.mhdgpu_batch_run_host(None, fake, fake, 1, None) == mhdgpu.MHD_ERR_ARG


def test_batch_arguments_rejected_without_a_gpu(L):
    import mhdgpu
    P = C.c_void_p
    h = P()
    good = [8, 8, 8, 32, 48, 64]
    fake = (P * 2)(P(0x1000), P(0x2000))
    dims = (C.c_int * 6)(*good)
    # axis outside 1 .. MHD_BATCH_MAX_PENCIL, no boxes, null tables, bad CFL
    bad = (C.c_int * 6)(8, 8, 8, 32, 257, 64)
    assert L.mhdgpu_batch_create(C.byref(h), 2, bad, fake, fake, 0.7, 0, None) == mhdgpu.MHD_ERR_ARG
    assert b"MHD_BATCH_MAX_PENCIL" in L.mhdgpu_last_error()
    assert L.mhdgpu_batch_create(C.byref(h), 0, dims, fake, fake, 0.7, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_batch_create(C.byref(h), 2, dims, None, fake, 0.7, 0, None) == mhdgpu.MHD_ERR_ARG
    nulls = (P * 2)(P(0x1000), None)
    assert L.mhdgpu_batch_create(C.byref(h), 2, dims, fake, nulls, 0.7, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_batch_create(C.byref(h), 2, dims, fake, fake, 0.0, 0, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_batch_create(C.byref(h), 2, dims, fake, fake, 0.7, 7, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_batch_create(None, 2, dims, fake, fake, 0.7, 0, None) == mhdgpu.MHD_ERR_ARG
    assert not h.value
    # calls on a null handle
    assert L.mhdgpu_batch_advance(None, 1, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_batch_set_schedule(None, 0, 128, 2) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_batch_destroy(None) == mhdgpu.MHD_ERR_ARG


def test_batch_workspace_bytes(L):
    import mhdgpu
    dims = [(8, 8, 8), (32, 48, 64)]
    cells = 8 ** 3 + 32 * 48 * 64
    ws = mhdgpu.batch_workspace_bytes(dims)
    assert 8 * cells < ws < 8 * cells + 4096
    assert mhdgpu.batch_workspace_bytes([(8, 8, 0)]) == 0
    assert mhdgpu.batch_workspace_bytes([(8, 300, 8)]) == 0


def test_diagnostics_arguments_without_a_gpu(L):
    import mhdgpu
    P = C.c_void_p
    fake = P(0x1000)
    assert L.mhdgpu_diagnostics_scratch_bytes(0, 4, 4) == 0
    assert 0 < L.mhdgpu_diagnostics_scratch_bytes(512, 512, 512) <= 40 * 1024
    assert L.mhdgpu_diagnostics(fake, fake, 0, 4, 4, fake, fake, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_diagnostics(None, fake, 4, 4, 4, fake, fake, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_diagnostics(fake, fake, 4, 4, 4, fake, None, None) == mhdgpu.MHD_ERR_ARG
    assert L.mhdgpu_set_math(mhdgpu.MHD_MATH_FP64P) == mhdgpu.MHD_MATH_FAITHFUL
    assert L.mhdgpu_set_math(mhdgpu.MHD_MATH_FAITHFUL) == mhdgpu.MHD_MATH_FP64P
    assert L.mhdgpu_set_math(3) == -1


def test_tile_cache_round_trip(L, tmp_path):
    """mhdgpu_tile_cache_save / _load: the shapes set in the table come back
    from the JSON file; a file recorded on another device model applies
    nothing; a malformed file is an argument error."""
    import json
    import mhdgpu
    f, r = mhdgpu.KCLASS["fluidx"], mhdgpu.KCLASS["fluidx"] | 16
    assert L.mhdgpu_set_tile(f, 200, 4, 2, 1) == 0
    assert L.mhdgpu_set_tile(r, 64, 2, 1, 8) == 0
    p = tmp_path / "tiles.json"
    mhdgpu.tile_cache_save(str(p))
    rec = json.load(open(p))
    assert rec["format"] == "mhdgpu tile cache 1"
    assert {"kclass": f, "n": 200, "cpl": 4, "wpp": 2, "ppc": 1} in rec["tiles"]
    assert L.mhdgpu_set_tile(f, 200, 2, 4, 1) == 0                        # changed after the save
    assert mhdgpu.tile_cache_load(str(p)) == len(rec["tiles"])
    assert mhdgpu.get_tile("fluidx", 200) == (4, 2, 1)
    assert mhdgpu.get_tile("fluidx", 64, rows=True) == (2, 1, 8)
    other = dict(rec, device="some other GPU")
    q = tmp_path / "other.json"
    json.dump(other, open(q, "w"))
    if rec["device"]:
        assert mhdgpu.tile_cache_load(str(q)) == 0
    bad = tmp_path / "bad.json"
    bad.write_text('{"format": "mhdgpu tile cache 1", "device": "", "tiles": [{"kclass": 0, "n": }]}')
    with pytest.raises(mhdgpu.MhdError):
        mhdgpu.tile_cache_load(str(bad))
    with pytest.raises(mhdgpu.MhdError):
        mhdgpu.tile_cache_load(str(tmp_path / "missing.json"))
