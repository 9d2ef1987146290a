"""PI state checkpoints in the reference's ":pid" format (checkpoints.jl); host only."""
import struct

import numpy as np
import pytest

import picuda


def _state(N=5, sectors=None, seed=0):
    b = picuda.PIBasis(N, 2, sectors=sectors)
    rng = np.random.default_rng(seed)
    return picuda.PIState(b, rng.standard_normal(len(b)) + 1j * rng.standard_normal(len(b)))


def test_round_trip_and_layout(tmp_path):
    st = _state(5, sectors=[(5, 0), (3, 2)])
    p = tmp_path / "s.pid"
    picuda.save_checkpoint(p, st, time=0.25, metadata={"model": "test", "N": 5})
    ck = picuda.load_checkpoint(p)
    assert ck.schema_version == picuda.PI_CHECKPOINT_VERSION and ck.time == 0.25
    assert ck.metadata == {"N": "5", "model": "test"}
    assert ck.state.basis.sectors == [(5, 0), (3, 2)]
    assert np.array_equal(ck.state.data, st.data)
    assert np.array_equal(picuda.checkpoint_state(ck).data, st.data)
    # byte layout of checkpoints.jl:111-134 (little-endian)
    raw = p.read_bytes()
    head = b"PIDCHKPT" + struct.pack("<HB", 1, 64) + struct.pack("<qii", 5, 2, 2) + struct.pack("<4q", 5, 0, 3, 2)
    head += struct.pack("<Bd", 1, 0.25) + struct.pack("<q", len(st.data))
    assert raw.startswith(head)
    body = raw[len(head):len(head) + 16 * len(st.data)]
    assert np.array_equal(np.frombuffer(body, "<f8"), st.data.view(np.float64))
    tail = struct.pack("<i", 2) + struct.pack("<I", 1) + b"N" + struct.pack("<I", 1) + b"5"
    tail += struct.pack("<I", 5) + b"model" + struct.pack("<I", 4) + b"test"
    assert raw[len(head) + 16 * len(st.data):] == tail


def test_float32_checkpoint_loads(tmp_path):
    """A Float32 checkpoint written in the same schema (scalar code 32) loads."""
    b = picuda.PIBasis(1, 2)
    vals = np.array([1.5, -2.0, 0.25, 3.0, 0.0, 1.0, -1.0, 0.5], dtype="<f4")
    raw = b"PIDCHKPT" + struct.pack("<HB", 1, 32) + struct.pack("<qii", 1, 2, 1) + struct.pack("<2q", 1, 0)
    raw += struct.pack("<B", 0) + struct.pack("<q", len(b)) + vals.tobytes() + struct.pack("<i", 0)
    p = tmp_path / "f32.pid"
    p.write_bytes(raw)
    ck = picuda.load_checkpoint(p)
    assert ck.time is None and ck.metadata == {}
    assert np.array_equal(ck.state.data, vals[0::2].astype(np.float64) + 1j * vals[1::2].astype(np.float64))


def test_invalid_checkpoints_raise(tmp_path):
    st = _state(3)
    p = tmp_path / "ok.pid"
    picuda.save_checkpoint(p, st)
    good = p.read_bytes()
    cases = {"magic": b"XXXXXXXX" + good[8:], "version": good[:8] + struct.pack("<H", 2) + good[10:],
             "trailing": good + b"\0", "truncated": good[:-3],
             "dup": good[:-4] + struct.pack("<i", 2) + (struct.pack("<I", 1) + b"k") * 4}
    for name, raw in cases.items():
        q = tmp_path / f"{name}.pid"
        q.write_bytes(raw)
        with pytest.raises((picuda.PiArgumentError, picuda.PiDimensionMismatch)):
            picuda.load_checkpoint(q)
    with pytest.raises(picuda.PiArgumentError):
        picuda.load_checkpoint(tmp_path / "missing.pid")
    with pytest.raises(picuda.PiArgumentError):
        picuda.save_checkpoint(tmp_path / "x.jld2", st)
    with pytest.raises(picuda.PiArgumentError):
        picuda.PIStateCheckpoint(st, time=float("inf"))
