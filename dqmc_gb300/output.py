"""Output files in the reference's JLD/HDF5 layout.

The reference writes, into its `.out.h5.running` file:

* `thermal_init/conf` (the field, `Array{Float64,3}` (3, N, M)) and
  `thermal_init/prethermalized` (the number of thermalisation ud-sweeps done)
  through JLD (`_save_thermal`, src/dqmc_framework.jl:322-333);
* `obs/configurations`, the measured fields, through MonteCarloObservable's
  on-disk observable (src/dqmc_framework.jl:406, 433-437, 456-457, 492): a
  group with `count` and the time series in chunks of `alloc` fields.

`write_thermal` and `ConfigurationWriter` write the same groups and datasets
so that a GPU run feeds the reference's own readers (`app/dqmc.jl:138-144`,
`src/measure_framework.jl:292, 443` via `loadobs_frommemory`).  The file is
an HDF5 file behind JLD's 512-byte header "Julia data file (HDF5), version
0.1.2", as in the reference's `test/data/*.jld`:

* superblock version 0 with base address 512 (the header is the user block);
* version-1 object headers; groups in compact "new style" storage (link-info,
  group-info and one link message per member);
* numeric datasets with the encodings of `test/data/O3.jld`: Float64
  (IEEE little-endian, 8 bytes), Int64 (signed, 8 bytes), UInt32; Julia's
  column-major array (d1, ..., dk) stored as the HDF5 dataspace (dk, ..., d1);
  fixed-length UTF-8 strings;
* the `_creator` group JLD writes (JULIA_MAJOR/MINOR/PATCH as UInt32,
  WORD_SIZE as Int64, ENDIAN_BOM as UInt32).

MonteCarloObservable's on-disk observable (version 0.3, not part of the
reference tree) is written as: `<group>/name`, `alloc`, `elsize` (Int64
vector), `eltype` (string), `count`, `timeseries/chunk_count` and
`timeseries/ts_chunk<i>` (Float64, the element dimensions followed by the
chunk's time index, (3, N, M, alloc) for the field).  `thermal_init/udsweep`
(a TimerOutputs object of the reference host's wall clock) has no counterpart
here and is not written.

The whole file is rewritten on each write (atomic rename), which suits the
sizes involved (one field is 1.2 MB at L=16, M=200).
"""
from __future__ import annotations

import os
import struct

import numpy as np

JLD_HEADER = b"Julia data file (HDF5), version 0.1.2"
USERBLOCK = 512
UNDEF = 0xFFFFFFFFFFFFFFFF

# Datatype messages (HDF5 datatype message version 1) with the encodings of the
# reference's JLD files.
_DT_F64 = bytes([0x11, 0x20, 0x3F, 0x00]) + struct.pack("<I", 8) + struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52,
                                                                                1023)
_DT_I64 = bytes([0x10, 0x08, 0x00, 0x00]) + struct.pack("<I", 8) + struct.pack("<HH", 0, 64)
_DT_U32 = bytes([0x10, 0x00, 0x00, 0x00]) + struct.pack("<I", 4) + struct.pack("<HH", 0, 32)
_FILL = bytes([0x02, 0x01, 0x02, 0x01, 0x00, 0x00, 0x00, 0x00])


def _dt_string(nbytes):
    # class 3 (string), version 1; null-terminated, UTF-8
    return bytes([0x13, 0x10, 0x00, 0x00]) + struct.pack("<I", nbytes)


def _pad8(b):
    return b + b"\0" * ((-len(b)) % 8)


class _Dataset:
    def __init__(self, dtype_msg, dims, raw):
        self.dtype_msg, self.dims, self.raw = dtype_msg, dims, raw


def _dataset_for(value):
    """(datatype message, HDF5 dims, raw bytes) of a Python/numpy value in JLD's
    encoding (Julia column-major arrays -> reversed HDF5 dims)."""
    if isinstance(value, str):
        b = value.encode("utf-8") + b"\0"
        return _Dataset(_dt_string(len(b)), (), b)
    if isinstance(value, (bool, np.bool_)):
        raise TypeError("booleans are not part of this layout")
    if isinstance(value, (int, np.integer)):
        return _Dataset(_DT_I64, (), struct.pack("<q", int(value)))
    if isinstance(value, (float, np.floating)):
        return _Dataset(_DT_F64, (), struct.pack("<d", float(value)))
    a = np.asarray(value)
    if a.dtype.kind == "f":
        dt, a = _DT_F64, a.astype("<f8")
    elif a.dtype.kind in "iu":
        dt, a = _DT_I64, a.astype("<i8")
    else:
        raise TypeError(f"unsupported array type {a.dtype}")
    return _Dataset(dt, tuple(reversed(a.shape)), a.tobytes(order="F"))


class _Writer:
    """Lays out a tree {name: subtree | _Dataset} as an HDF5 file."""

    def __init__(self):
        self.buf = bytearray()

    def alloc(self, nbytes):
        addr = len(self.buf)
        self.buf += b"\0" * nbytes
        return addr

    def put(self, addr, data):
        self.buf[addr:addr + len(data)] = data

    @staticmethod
    def _msg(mtype, body, flags=0):
        body = _pad8(body)
        return struct.pack("<HHB3x", mtype, len(body), flags) + body

    def _object_header(self, messages):
        body = b"".join(messages)
        hdr = struct.pack("<BxHII4x", 1, len(messages), 1, len(body))
        addr = self.alloc(len(hdr) + len(body))
        self.put(addr, hdr + body)
        return addr

    def dataset(self, ds):
        rank = len(ds.dims)
        space = struct.pack("<BBBx4x", 1, rank, 0) + b"".join(struct.pack("<Q", d) for d in ds.dims)
        if len(ds.raw) <= 512:
            layout = struct.pack("<BBH", 3, 0, len(ds.raw)) + ds.raw          # compact
            data_addr = None
        else:
            data_addr = self.alloc(len(ds.raw))                              # contiguous
            self.put(data_addr, ds.raw)
            layout = struct.pack("<BBQQ", 3, 1, data_addr, len(ds.raw))
        msgs = [self._msg(0x0001, space), self._msg(0x0003, ds.dtype_msg, flags=1),
                self._msg(0x0005, _FILL, flags=1), self._msg(0x0008, layout)]
        return self._object_header(msgs)

    def group(self, tree):
        links = []
        for name in sorted(tree):
            child = tree[name]
            addr = self.group(child) if isinstance(child, dict) else self.dataset(child)
            nm = name.encode("utf-8")
            if len(nm) > 255:
                raise ValueError("link name too long")
            # link message v1: flags 0x10 (charset present), UTF-8, 1-byte name length, hard link
            links.append(self._msg(0x0006, struct.pack("<BBBB", 1, 0x10, 1, len(nm)) + nm + struct.pack("<Q", addr)))
        linfo = struct.pack("<BBQQ", 0, 0, UNDEF, UNDEF)
        ginfo = struct.pack("<BB", 0, 0)
        return self._object_header([self._msg(0x0002, linfo), self._msg(0x000A, ginfo, flags=1)] + links)

    def file(self, tree):
        self.alloc(96)                      # superblock v0 with the root symbol-table entry
        root = self.group(tree)
        sb = bytearray(96)
        sb[0:8] = b"\x89HDF\r\n\x1a\n"
        sb[8:16] = bytes([0, 0, 0, 0, 0, 8, 8, 0])
        struct.pack_into("<HHI", sb, 16, 4, 16, 0)
        struct.pack_into("<QQQQ", sb, 24, USERBLOCK, UNDEF, USERBLOCK + len(self.buf), UNDEF)
        struct.pack_into("<QQII", sb, 56, 0, root, 0, 0)
        self.put(0, bytes(sb))
        head = JLD_HEADER + b"\0" * (USERBLOCK - len(JLD_HEADER))
        return head + bytes(self.buf)


def _creator():
    # JLD's `_creator` group; the Julia version fields name the reference's CI version (1.3.1)
    return {"JULIA_MAJOR": _Dataset(_DT_U32, (), struct.pack("<I", 1)),
            "JULIA_MINOR": _Dataset(_DT_U32, (), struct.pack("<I", 3)),
            "JULIA_PATCH": _Dataset(_DT_U32, (), struct.pack("<I", 1)),
            "WORD_SIZE": _Dataset(_DT_I64, (), struct.pack("<q", 64)),
            "ENDIAN_BOM": _Dataset(_DT_U32, (), struct.pack("<I", 0x04030201))}


def _insert(tree, path, value):
    parts = [p for p in path.split("/") if p]
    node = tree
    for p in parts[:-1]:
        node = node.setdefault(p, {})
        if not isinstance(node, dict):
            raise ValueError(f"{path}: {p} is a dataset")
    node[parts[-1]] = value if isinstance(value, (_Dataset, dict)) else _dataset_for(value)


class JLDFile:
    """An output file held as a tree of datasets and written whole on save()."""

    def __init__(self, path):
        self.path = path
        self.tree = {"_creator": _creator()}

    def __setitem__(self, name, value):
        _insert(self.tree, name, value)

    def __contains__(self, name):
        node = self.tree
        for p in [p for p in name.split("/") if p]:
            if not isinstance(node, dict) or p not in node:
                return False
            node = node[p]
        return True

    def save(self):
        data = _Writer().file(self.tree)
        tmp = self.path + ".tmp"
        with open(tmp, "wb") as f:
            f.write(data)
        os.replace(tmp, self.path)


def write_thermal(jf: JLDFile, conf, prethermalized: int, box: float | None = None):
    """`_save_thermal` (src/dqmc_framework.jl:322-333): the field (3, N, M) and
    the number of thermalisation ud-sweeps done; `box` as
    `thermal_init/box` (read back by app/dqmc.jl:146-149) when given."""
    conf = np.asarray(conf, dtype=np.float64)
    if conf.ndim != 3 or conf.shape[0] != 3:
        raise ValueError("conf must have shape (3, N, M)")
    jf["thermal_init/conf"] = conf
    jf["thermal_init/prethermalized"] = int(prethermalized)
    if box is not None:
        jf["thermal_init/box"] = float(box)
    jf.save()


class ConfigurationWriter:
    """The on-disk observable `obs/configurations` (src/dqmc_framework.jl:406):
    push!(field) buffers, every `alloc` fields form one chunk, flush() writes
    the partial chunk (src/dqmc_framework.jl:433-437, 456-457, 492)."""

    def __init__(self, jf: JLDFile, alloc: int, group: str = "obs/configurations", name: str = "configurations"):
        self.jf, self.alloc, self.group, self.name = jf, int(alloc), group.rstrip("/"), name
        self.buf = []
        self.chunks = 0
        self.count = 0
        self.elsize = None

    def push(self, conf):
        conf = np.array(conf, dtype=np.float64)
        if self.elsize is None:
            self.elsize = conf.shape
        elif conf.shape != self.elsize:
            raise ValueError("all configurations must have the same shape")
        self.buf.append(conf)
        self.count += 1
        if len(self.buf) == self.alloc:
            self._write_chunk()

    def _write_chunk(self):
        if not self.buf:
            return
        self.chunks += 1
        ts = np.stack(self.buf, axis=-1)          # element dims, then the time index
        g = self.group
        self.jf[f"{g}/timeseries/ts_chunk{self.chunks}"] = ts
        self.jf[f"{g}/timeseries/chunk_count"] = self.chunks
        self.jf[f"{g}/name"] = self.name
        self.jf[f"{g}/alloc"] = self.alloc
        self.jf[f"{g}/elsize"] = np.asarray(self.elsize, dtype=np.int64)
        self.jf[f"{g}/eltype"] = f"Array{{Float64,{len(self.elsize)}}}"
        self.jf[f"{g}/count"] = self.count
        self.buf = []
        self.jf.save()

    def flush(self):
        self._write_chunk()
