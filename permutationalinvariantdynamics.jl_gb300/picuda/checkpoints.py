"""Versioned PI state checkpoints (checkpoints.jl), byte-compatible with the reference's
dependency-free ":pid" format, so a state saved by either side loads in the other.

Layout (little-endian, checkpoints.jl:111-134): magic "PIDCHKPT"; UInt16 schema version 1;
UInt8 scalar code (16, 32, 64 = Float16/32/64); Int64 N; Int32 d; Int32 sector count; per
sector d Int64 partition parts; UInt8 time flag [+ one real]; Int64 coefficient count; the
coefficients as (real, imag) pairs; Int32 metadata count; per entry (sorted by key) a UInt32
length-prefixed UTF-8 key and value.  BigFloat checkpoints (code 128) are not produced or
read here: the CUDA path's states are FP64.

A state may be a PIState or a CUDA tensor of complex128 coefficients with its basis (the
resident states of a solve or of the serving loop); saving copies it to the host once.
"""
from __future__ import annotations

import os
import struct
from dataclasses import dataclass, field

import numpy as np

from ._lib import PiArgumentError, PiDimensionMismatch
from .core import PIBasis, PIState

PI_CHECKPOINT_VERSION = 1
_MAGIC = b"PIDCHKPT"
_CODES = {16: np.float16, 32: np.float32, 64: np.float64}


@dataclass
class PIStateCheckpoint:
    """PIStateCheckpoint(state; time, metadata) (checkpoints.jl:15-40)."""
    state: PIState
    time: float | None = None
    metadata: dict = field(default_factory=dict)
    schema_version: int = PI_CHECKPOINT_VERSION

    def __post_init__(self):
        if self.time is not None:
            if isinstance(self.time, bool) or not isinstance(self.time, (int, float, np.floating, np.integer)):
                raise PiArgumentError("checkpoint time must be real")
            converted = float(self.time)
            if not np.isfinite(converted):
                raise PiArgumentError("checkpoint time is not finite in state precision Float64")
            if converted != self.time:
                raise PiArgumentError("checkpoint time cannot be represented exactly in state precision Float64")
            self.time = converted
        self.metadata = {str(k): str(v) for k, v in dict(self.metadata).items()}
        self.state = PIState(self.state.basis, np.array(self.state.data, dtype=np.complex128))


def checkpoint_state(checkpoint: PIStateCheckpoint) -> PIState:
    """A detached copy of the stored state (checkpoints.jl:43)."""
    return checkpoint.state.copy()


def _format(path, fmt):
    """checkpoints.jl:45-51."""
    if fmt != "auto":
        return fmt
    ext = os.path.splitext(str(path))[1].lower()
    if ext in (".jld2", ".jld"):
        return "jld2"
    if ext in (".h5", ".hdf5"):
        return "hdf5"
    return "pid"


def _as_state(state, basis):
    if isinstance(state, PIState):
        return state
    if basis is None:
        raise PiArgumentError("a device state needs its basis")
    data = state.detach().cpu().numpy() if hasattr(state, "detach") else np.asarray(state)
    return PIState(basis, np.asarray(data, dtype=np.complex128))


def _write_string(out, value):
    b = value.encode("utf-8")
    if len(b) > 0xFFFFFFFF:
        raise PiArgumentError("checkpoint string is too long")
    out += struct.pack("<I", len(b)) + b


def save_checkpoint(path, checkpoint_or_state, time=None, metadata=None, format="auto", basis=None):
    """save_checkpoint(path, checkpoint | state; time, metadata, format) (checkpoints.jl:193-213)."""
    if isinstance(checkpoint_or_state, PIStateCheckpoint):
        ck = checkpoint_or_state
    else:
        ck = PIStateCheckpoint(_as_state(checkpoint_or_state, basis), time, metadata or {})
    if ck.schema_version != PI_CHECKPOINT_VERSION:
        raise PiArgumentError(f"cannot write unsupported checkpoint schema {ck.schema_version}")
    fmt = _format(path, format)
    if fmt in ("jld2", "hdf5"):
        raise PiArgumentError(f"checkpoint format :{fmt} requires loading the corresponding optional JLD2 or HDF5 package")
    if fmt != "pid":
        raise PiArgumentError(f"unknown PI checkpoint format :{fmt}")
    b = ck.state.basis
    out = bytearray(_MAGIC)
    out += struct.pack("<HB", ck.schema_version, 64)
    out += struct.pack("<qii", b.N, b.d, len(b.sectors))
    for parts in b.sectors:
        out += struct.pack(f"<{len(parts)}q", *parts)
    out += struct.pack("<B", 0 if ck.time is None else 1)
    if ck.time is not None:
        out += struct.pack("<d", ck.time)
    data = np.ascontiguousarray(ck.state.data, dtype=np.complex128)
    out += struct.pack("<q", len(data))
    out += data.view(np.float64).astype("<f8").tobytes()
    out += struct.pack("<i", len(ck.metadata))
    for key in sorted(ck.metadata):
        _write_string(out, key)
        _write_string(out, ck.metadata[key])
    with open(path, "wb") as f:
        f.write(out)
    return str(path)


class _Reader:
    def __init__(self, buf):
        self.buf, self.pos = buf, 0

    def take(self, fmt):
        size = struct.calcsize(fmt)
        if self.pos + size > len(self.buf):
            raise PiArgumentError("truncated PI checkpoint")
        vals = struct.unpack_from(fmt, self.buf, self.pos)
        self.pos += size
        return vals if len(vals) > 1 else vals[0]

    def string(self):
        n = self.take("<I")
        if n > len(self.buf) - self.pos:
            raise PiArgumentError("checkpoint string length exceeds the remaining file payload")
        s = self.buf[self.pos:self.pos + n].decode("utf-8")
        self.pos += n
        return s


def load_checkpoint(path, format="auto") -> PIStateCheckpoint:
    """load_checkpoint(path; format) (checkpoints.jl:224-232, reader :136-182)."""
    if not os.path.isfile(path):
        raise PiArgumentError(f"checkpoint file does not exist: {path}")
    fmt = _format(path, format)
    if fmt != "pid":
        raise PiArgumentError(f"checkpoint format :{fmt} requires loading the corresponding optional JLD2 or HDF5 package")
    with open(path, "rb") as f:
        r = _Reader(f.read())
    if r.buf[:8] != _MAGIC:
        raise PiArgumentError("file is not a PI checkpoint")
    r.pos = 8
    version = r.take("<H")
    if version != PI_CHECKPOINT_VERSION:
        raise PiArgumentError(f"unsupported PI checkpoint schema version {version}")
    code = r.take("<B")
    if code == 128:
        raise PiArgumentError("BigFloat checkpoints are outside the CUDA path (FP64 states)")
    if code not in _CODES:
        raise PiArgumentError(f"unknown PI checkpoint scalar code {code}")
    rtype = np.dtype(_CODES[code]).newbyteorder("<")
    N, d, ns = r.take("<q"), r.take("<i"), r.take("<i")
    if not (N >= 0 and d >= 1 and ns >= 1):
        raise PiArgumentError("invalid PI checkpoint basis metadata")
    sectors = [tuple(int(v) for v in np.atleast_1d(r.take(f"<{d}q"))) for _ in range(ns)]
    basis = PIBasis(N, d, sectors=sectors)
    has_time = r.take("<B")
    if has_time not in (0, 1):
        raise PiArgumentError("invalid PI checkpoint time flag")
    time = float(r.take(f"<{rtype.char}")) if has_time else None
    count = r.take("<q")
    if count != len(basis):
        raise PiDimensionMismatch("PI checkpoint coefficient length does not match its basis")
    nbytes = 2 * count * rtype.itemsize
    if r.pos + nbytes > len(r.buf):
        raise PiArgumentError("truncated PI checkpoint")
    raw = np.frombuffer(r.buf, dtype=rtype, count=2 * count, offset=r.pos).astype(np.float64)
    r.pos += nbytes
    data = raw[0::2] + 1j * raw[1::2]
    nmeta = r.take("<i")
    if nmeta < 0:
        raise PiArgumentError("invalid PI checkpoint metadata count")
    metadata = {}
    for _ in range(nmeta):
        key = r.string()
        if key in metadata:
            raise PiArgumentError(f"duplicate PI checkpoint metadata key {key}")
        metadata[key] = r.string()
    if r.pos != len(r.buf):
        raise PiArgumentError("trailing data in PI checkpoint")
    return PIStateCheckpoint(PIState(basis, data), time, metadata, version)
