"""Checkpoint and snapshot files in the reference's format (escreve_par.f).

The files are gfortran sequential unformatted: records framed by 4-byte
length markers, long records split into subrecords with negated markers.
This test reads and writes them with its own implementation of that layout
and checks the library against it, byte for byte.
"""
import struct

import numpy as np
import pytest

from tests.helpers import NAMES, perturbed_state, small_case

pytestmark = pytest.mark.gpu


def read_records(path):
    data = open(path, "rb").read()
    recs, pos = [], 0
    while pos < len(data):
        parts, first = [], True
        while True:
            head = struct.unpack("<i", data[pos:pos + 4])[0]
            n = abs(head)
            parts.append(data[pos + 4:pos + 4 + n])
            tail = struct.unpack("<i", data[pos + 4 + n:pos + 8 + n])[0]
            assert abs(tail) == n
            assert (tail < 0) == (not first), "trailing marker sign"
            pos += 8 + n
            first = False
            if head >= 0:
                break
        recs.append((b"".join(parts), len(parts)))
    return recs


def write_records(path, payloads):
    with open(path, "wb") as f:
        for p in payloads:
            f.write(struct.pack("<i", len(p)) + p + struct.pack("<i", len(p)))


def state_bytes(st):
    return b"".join(np.ascontiguousarray(st[n], dtype=np.complex128).tobytes() for n in NAMES)


@pytest.fixture(scope="module")
def ctx():
    from trans_bl_gb300 import api
    cfg, coefs, base = small_case()
    g = api.Context(cfg, coefs, base)
    st = perturbed_state(cfg, base, np.random.default_rng(41))
    g.put_state(st)
    return g, cfg, coefs, base, api


def test_checkpoint_layout(ctx, tmp_path):
    g, cfg, coefs, base, api = ctx
    p = tmp_path / "data_00.bin"
    g.write_checkpoint(p, 1234)
    recs = read_records(p)
    assert len(recs) == 2
    assert struct.unpack("<i", recs[0][0])[0] == 1234
    assert recs[1][0] == state_bytes(g.get_state())


def test_checkpoint_restart(ctx, tmp_path):
    g, cfg, coefs, base, api = ctx
    st = g.get_state()
    p = tmp_path / "data_00.bin"
    write_records(p, [struct.pack("<i", 77), state_bytes(st)])   # as the Fortran host writes it
    h = api.Context(cfg, coefs, base)
    assert h.read_checkpoint(p) == 77
    back = h.get_state()
    for n in NAMES:
        assert np.array_equal(back[n], st[n]), n
    h.close()


def test_subrecords(ctx, tmp_path):
    g, cfg, coefs, base, api = ctx
    p = tmp_path / "data_00.bin"
    api.check(api.load().tb_io_set_subrecord_limit(1000), "limit")
    try:
        g.write_checkpoint(p, 5)
    finally:
        api.check(api.load().tb_io_set_subrecord_limit(2147483639), "limit")
    recs = read_records(p)
    n = len(state_bytes(g.get_state()))
    assert recs[1][1] == -(-n // 1000)          # number of subrecords
    assert recs[1][0] == state_bytes(g.get_state())
    h = api.Context(cfg, coefs, base)
    assert h.read_checkpoint(p) == 5
    assert np.array_equal(h.get_state()["wz"], g.get_state()["wz"])
    h.close()


def test_pert_snapshot(ctx, tmp_path):
    g, cfg, coefs, base, api = ctx
    p = tmp_path / "pert_00_01"
    g.write_pert(p)
    recs = read_records(p)
    assert len(recs) == 1
    ux = np.frombuffer(recs[0][0], dtype=np.complex128).reshape(cfg.kfour, cfg.ny, cfg.nx)
    want = g.get_state()["ux"].copy()
    want[0] = want[0] - base[0]
    assert np.array_equal(ux, want)


def test_bad_files(ctx, tmp_path):
    g, cfg, coefs, base, api = ctx
    st = g.get_state()
    p = tmp_path / "short.bin"
    write_records(p, [struct.pack("<i", 1), state_bytes(st)[:-16]])   # one element short
    with pytest.raises(api.TbError):
        g.read_checkpoint(p)
    q = tmp_path / "trunc.bin"
    q.write_bytes(p.read_bytes()[:100])
    with pytest.raises(api.TbError):
        g.read_checkpoint(q)
