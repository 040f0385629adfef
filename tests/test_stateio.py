"""CPU tests of the state files in the reference's formats (mhdgpu_read_state,
mhdgpu_write_state, mhdgpu_write_result, mhdgpu_write_check): host code of the
library, no GPU needed.

Pinning: writing the reference's shipped 16^3 Alfven state (decoded into the
golden fixture alfven16_dat.npz) reproduces the shipped file byte for byte
(its sha256, recorded by tests/golden/gen_golden.py), and reading that file
back gives the state the reference's init.c reads."""
import hashlib
import os

import numpy as np
import pytest

from util import bits_equal

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def M():
    import mhdgpu
    if not os.path.exists(mhdgpu.LIB_PATH):
        import build
        build.build()
    mhdgpu.lib()
    return mhdgpu


def coded_state(nx, ny, nz):
    """u, b whose every value encodes (field, i, j, k)."""
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    code = (i + 100 * j + 10000 * k).astype(np.float64)
    u = np.stack([code + 0.1 * (f + 1) for f in range(5)], axis=-1).astype(np.float32).ravel()
    b = np.stack([code + 0.1 * (f + 6) for f in range(3)], axis=-1).astype(np.float32).ravel()
    return u, b


def test_state_file_layout_x_outer_z_inner(M, tmp_path):
    nx, ny, nz = 5, 3, 4
    u, b = coded_state(nx, ny, nz)
    p = tmp_path / "s.dat"
    M.write_state(str(p), u, b, nx, ny, nz)
    raw = np.fromfile(p, dtype=np.float32).reshape(nx, ny, nz, 8)    # file: i, j, k, field
    uu = u.reshape(nz, ny, nx, 5).transpose(2, 1, 0, 3)
    bb = b.reshape(nz, ny, nx, 3).transpose(2, 1, 0, 3)
    assert bits_equal(raw[..., :5].copy(), uu.copy()) and bits_equal(raw[..., 5:].copy(), bb.copy())
    u2, b2 = M.read_state(str(p), nx, ny, nz)
    assert bits_equal(u2, u) and bits_equal(b2, b)


def test_state_file_matches_reference_shipped_file(M, tmp_path):
    g = np.load(os.path.join(GOLD, "alfven16_dat.npz"))
    digest, size = open(os.path.join(GOLD, "alfven16_dat_sha256.txt")).read().split()
    p = tmp_path / "alfven16.dat"
    M.write_state(str(p), g["u0"], g["b0"], 16, 16, 16)
    raw = p.read_bytes()
    assert len(raw) == int(size) and hashlib.sha256(raw).hexdigest() == digest
    u, b = M.read_state(str(p), 16, 16, 16)
    assert bits_equal(u, g["u0"]) and bits_equal(b, g["b0"])


def test_result_dump_layout(M, tmp_path):
    nx, ny, nz = 4, 6, 3
    u, b = coded_state(nx, ny, nz)
    pu, pb = tmp_path / "result_u1.dat", tmp_path / "result_b1.dat"
    M.write_result(str(pu), str(pb), u, b, nx, ny, nz)
    ru = np.fromfile(pu, dtype=np.float32).reshape(nx, ny, nz, 5)
    rb = np.fromfile(pb, dtype=np.float32).reshape(nx, ny, nz, 3)
    assert bits_equal(ru, u.reshape(nz, ny, nx, 5).transpose(2, 1, 0, 3).copy())
    assert bits_equal(rb, b.reshape(nz, ny, nx, 3).transpose(2, 1, 0, 3).copy())


def test_check_dump_text(M, tmp_path):
    import ics
    nx, ny, nz = 6, 4, 5
    u, b = ics.random_state(nx, ny, nz, seed=2)
    prefix = str(tmp_path / "C_version_check_")
    M.write_check(prefix, u, b, nx, ny, nz)
    for f, name in enumerate(("u1", "u2", "u3", "u4", "u5", "b1", "b2", "b3")):
        lines = open(prefix + name + ".dat").read().splitlines()
        src = u.reshape(-1, 5)[:, f] if f < 5 else b.reshape(-1, 3)[:, f - 5]
        assert lines == ["%8.6e" % float(v) for v in src], name


def test_state_file_errors(M, tmp_path):
    u, b = coded_state(4, 4, 4)
    p = tmp_path / "s.dat"
    M.write_state(str(p), u, b, 4, 4, 4)
    with pytest.raises(M.MhdError) as ei:
        M.read_state(str(p), 4, 4, 5)                 # wrong size
    assert ei.value.status == M.MHD_ERR_ARG
    with pytest.raises(M.MhdError) as ei:
        M.read_state(str(tmp_path / "missing.dat"), 4, 4, 4)
    assert ei.value.status == M.MHD_ERR_NOMEM
    with pytest.raises(ValueError):
        M.write_state(str(p), u.astype(np.float64), b, 4, 4, 4)
