"""Minimal read-only HDF5 reader for the reference's JLD 0.1.2 golden files.

Neither h5py nor libhdf5 is available, so this module decodes the small
subset of the HDF5 file format (public specification, "HDF5 File Format
Specification Version 3.0") that the reference's `test/data/*.jld` files use:

  * superblock version 0 behind the 512-byte JLD user block;
  * version-1 object headers with continuation blocks;
  * "new style" groups: link-info message -> fractal heap + version-2 B-tree
    (type-5 name records), and "old style" groups (symbol table message ->
    version-1 B-tree + SNOD nodes + local heap);
  * datasets with compact or contiguous layout;
  * datatypes: fixed-point, floating-point, compound (version 1 and 3),
    object references, committed (shared) datatypes;
  * JLD's encoding of `Complex{Float64}` (compound re/im) and of
    `SparseMatrixCSC` (compound m, n, colptr, rowval, nzval with object
    references for the arrays).

It is a fixture-generation tool: only `tests/golden/make_golden.py` uses it.
Arrays are returned in the reference's (Julia, column-major) index order.
"""
from __future__ import annotations

import struct

import numpy as np
import scipy.sparse as sps


class _Reader:
    def __init__(self, path):
        self.d = open(path, "rb").read()
        self.base = self.d.find(b"\x89HDF\r\n\x1a\n")
        assert self.base >= 0, "no HDF5 signature"
        sb = self.d[self.base:self.base + 96]
        assert sb[8] == 0, "only superblock v0 is supported"
        self.so, self.sl = sb[13], sb[14]
        assert self.so == 8 and self.sl == 8
        root_entry = self.base + 56
        self.root = struct.unpack_from("<Q", self.d, root_entry + 8)[0]
        self._hdr_cache = {}

    # -- primitive access ----------------------------------------------------
    def abs(self, addr):
        return self.base + addr

    def u(self, fmt, off):
        return struct.unpack_from(fmt, self.d, off)

    # -- object headers --------------------------------------------------------
    def messages(self, addr):
        """List of (type, flags, bytes) of a version-1 object header."""
        if addr in self._hdr_cache:
            return self._hdr_cache[addr]
        off = self.abs(addr)
        ver = self.d[off]
        assert ver == 1, f"object header version {ver} unsupported"
        nmsg = self.u("<H", off + 2)[0]
        hsize = self.u("<I", off + 8)[0]
        blocks = [(off + 16, hsize)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(out) < nmsg:
                mtype, msize, mflags = self.u("<HHB", p)
                data = self.d[p + 8:p + 8 + msize]
                if mtype == 0x10:            # continuation
                    caddr, clen = struct.unpack_from("<QQ", data, 0)
                    blocks.append((self.abs(caddr), clen))
                out.append((mtype, mflags, data))
                p += 8 + msize
        self._hdr_cache[addr] = out
        return out

    # -- groups ------------------------------------------------------------------
    def links(self, addr):
        """name -> object header address for the group at `addr`."""
        res = {}
        for mtype, _, data in self.messages(addr):
            if mtype == 0x02:                # link info
                flags = data[1]
                p = 2 + (8 if flags & 1 else 0)
                heap, btree = struct.unpack_from("<QQ", data, p)
                if heap != 0xFFFFFFFFFFFFFFFF:
                    res.update(self._dense_links(heap, btree))
            elif mtype == 0x06:              # compact link
                name, target = self._parse_link(data, 0)[:2]
                res[name] = target
            elif mtype == 0x11:              # symbol table (old style)
                btree, heap = struct.unpack_from("<QQ", data, 0)
                res.update(self._symtab_links(btree, heap))
        return res

    def _parse_link(self, d, p):
        ver, flags = d[p], d[p + 1]
        assert ver == 1
        p += 2
        ltype = 0
        if flags & 0x8:
            ltype = d[p]; p += 1
        if flags & 0x4:
            p += 8
        if flags & 0x10:
            p += 1
        nlen_size = 1 << (flags & 3)
        nlen = int.from_bytes(d[p:p + nlen_size], "little"); p += nlen_size
        name = d[p:p + nlen].decode("utf-8"); p += nlen
        assert ltype == 0, "only hard links supported"
        target = struct.unpack_from("<Q", d, p)[0]; p += 8
        return name, target, p

    def _fractal_heap(self, heap):
        off = self.abs(heap)
        assert self.d[off:off + 4] == b"FRHP"
        p = off + 5
        idlen, filtlen = self.u("<HH", p); p += 4
        hflags = self.d[p]; p += 1
        p += 4                                    # max managed object size
        p += 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8
        width = self.u("<H", p)[0]; p += 2
        start_block, max_direct = self.u("<QQ", p); p += 16
        max_heap_bits = self.u("<H", p)[0]; p += 2
        p += 2                                    # starting # rows
        root_addr = self.u("<Q", p)[0]; p += 8
        cur_rows = self.u("<H", p)[0]; p += 2
        assert filtlen == 0
        return dict(idlen=idlen, width=width, start_block=start_block, max_direct=max_direct,
                    max_heap_bits=max_heap_bits, root=root_addr, rows=cur_rows, addr=heap,
                    flags=hflags)

    def _heap_blocks(self, h):
        """List of (heap offset, file position, size) of the direct blocks."""
        off_bytes = (h["max_heap_bits"] + 7) // 8
        if h["rows"] == 0:
            return [(0, self.abs(h["root"]), h["start_block"])]
        blocks = []
        p = self.abs(h["root"])
        assert self.d[p:p + 4] == b"FHIB"
        p += 5 + 8 + off_bytes
        heap_off = 0
        size = h["start_block"]
        for row in range(h["rows"]):
            if row >= 2:
                size = h["start_block"] << (row - 1)
            for _ in range(h["width"]):
                if size > h["max_direct"]:
                    break
                baddr = self.u("<Q", p)[0]; p += 8
                if baddr != 0xFFFFFFFFFFFFFFFF:
                    blocks.append((heap_off, self.abs(baddr), size))
                heap_off += size
        return blocks

    def _heap_object(self, h, hid):
        off_bytes = (h["max_heap_bits"] + 7) // 8
        assert hid[0] & 0x30 == 0, "only managed heap objects supported"
        hoff = int.from_bytes(hid[1:1 + off_bytes], "little")
        len_bytes = min((h["max_direct"].bit_length() + 7) // 8, h["idlen"] - 1 - off_bytes)
        hlen = int.from_bytes(hid[1 + off_bytes:1 + off_bytes + len_bytes], "little")
        for boff, bpos, bsize in self._heap_blocks(h):
            if boff <= hoff < boff + bsize:
                return self.d[bpos + (hoff - boff):bpos + (hoff - boff) + hlen]
        raise KeyError("heap offset not found")

    def _dense_links(self, heap, btree):
        """Links of a dense-storage group: every managed object of the
        group's fractal heap is one link message, packed back to back at
        the start of each direct block (the name index B-tree is not
        needed to enumerate them)."""
        h = self._fractal_heap(heap)
        off_bytes = (h["max_heap_bits"] + 7) // 8
        hdr = 4 + 1 + 8 + off_bytes + (4 if h["flags"] & 0x2 else 0)
        res = {}
        for boff, bpos, bsize in self._heap_blocks(h):
            assert self.d[bpos:bpos + 4] == b"FHDB"
            blk = self.d[bpos:bpos + bsize]
            p = hdr
            while p + 2 < bsize and blk[p] == 1:
                name, target, p = self._parse_link(blk, p)
                res[name] = target
        return res

    def _symtab_links(self, btree, heap):
        hp = self.abs(heap)
        assert self.d[hp:hp + 4] == b"HEAP"
        data_addr = self.u("<Q", hp + 24)[0]
        res = {}

        def name_at(o):
            s = self.abs(data_addr) + o
            e = self.d.index(b"\x00", s)
            return self.d[s:e].decode()

        def walk(node):
            p = self.abs(node)
            assert self.d[p:p + 4] == b"TREE"
            ntype, level, used = self.d[p + 4], self.d[p + 5], self.u("<H", p + 6)[0]
            q = p + 24
            children = []
            for i in range(used):
                q += 8                               # key
                children.append(self.u("<Q", q)[0]); q += 8
            for c in children:
                if level > 0:
                    walk(c)
                else:
                    s = self.abs(c)
                    assert self.d[s:s + 4] == b"SNOD"
                    nsym = self.u("<H", s + 6)[0]
                    e = s + 8
                    for _ in range(nsym):
                        lno, oh = self.u("<QQ", e)
                        res[name_at(lno)] = oh
                        e += 40
        walk(btree)
        return res

    # -- datatypes -------------------------------------------------------------
    def datatype(self, data, p=0):
        """Parse a datatype message at data[p:]; returns (dtype-descr, size, end)."""
        cv = data[p]
        cls, ver = cv & 0x0F, cv >> 4
        bits = data[p + 1] | (data[p + 2] << 8) | (data[p + 3] << 16)
        size = struct.unpack_from("<I", data, p + 4)[0]
        q = p + 8
        if cls == 0:
            signed = bool(bits & 0x8)
            q += 4
            return ("int", size, signed), size, q
        if cls == 1:
            q += 12
            return ("float", size), size, q
        if cls == 7:
            return ("ref", size), size, q
        if cls == 3:
            return ("string", size), size, q
        if cls == 6:
            nmem = bits & 0xFFFF
            members = []
            for _ in range(nmem):
                e = data.index(b"\x00", q)
                name = data[q:e].decode()
                if ver < 3:
                    q = q + ((e - q + 1 + 7) // 8) * 8
                    moff = struct.unpack_from("<I", data, q)[0]
                    q += 4 + 1 + 3 + 4 + 4 + 16
                else:
                    q = e + 1
                    nb = max(1, (size.bit_length() + 7) // 8)
                    moff = int.from_bytes(data[q:q + nb], "little")
                    q += nb
                mt, msz, q = self.datatype(data, q)
                members.append((name, moff, mt, msz))
            return ("compound", size, members), size, q
        if cls == 9:                                 # variable length
            base, _, q2 = self.datatype(data, q)
            return ("vlen", size, base), size, q2
        raise NotImplementedError(f"datatype class {cls}")

    def _object_datatype(self, addr):
        for mtype, mflags, data in self.messages(addr):
            if mtype == 0x03:
                if mflags & 0x2:
                    return self._shared_datatype(data)
                return self.datatype(data)[0]
        raise KeyError("no datatype")

    def _shared_datatype(self, data):
        ver = data[0]
        if ver == 1:
            a = struct.unpack_from("<Q", data, 8)[0]
        else:
            a = struct.unpack_from("<Q", data, 2)[0]
        return self._object_datatype(a)

    # -- datasets ----------------------------------------------------------------
    def dataset(self, addr):
        dims, dtype, raw = None, None, None
        for mtype, mflags, data in self.messages(addr):
            if mtype == 0x01:
                ver, nd, fl = data[0], data[1], data[2]
                p = 8 if ver == 1 else 4
                dims = [struct.unpack_from("<Q", data, p + 8 * i)[0] for i in range(nd)]
                if ver == 2 and data[3] == 1:
                    dims = []                         # scalar
            elif mtype == 0x03:
                dtype = self._shared_datatype(data) if mflags & 0x2 else self.datatype(data)[0]
            elif mtype == 0x08:
                ver = data[0]
                assert ver == 3, f"layout version {ver}"
                lcls = data[1]
                if lcls == 0:
                    sz = struct.unpack_from("<H", data, 2)[0]
                    raw = data[4:4 + sz]
                elif lcls == 1:
                    a, sz = struct.unpack_from("<QQ", data, 2)
                    raw = b"" if a == 0xFFFFFFFFFFFFFFFF else self.d[self.abs(a):self.abs(a) + sz]
                else:
                    raise NotImplementedError("chunked layout")
        return dims, dtype, raw

    def _decode(self, dtype, raw, count):
        kind = dtype[0]
        if kind == "float":
            return np.frombuffer(raw, dtype="<f8" if dtype[1] == 8 else "<f4", count=count)
        if kind == "int":
            code = {(8, True): "<i8", (8, False): "<u8", (4, True): "<i4", (4, False): "<u4",
                    (1, True): "i1", (1, False): "u1"}[(dtype[1], dtype[2])]
            return np.frombuffer(raw, dtype=code, count=count)
        if kind == "ref":
            return np.frombuffer(raw, dtype="<u8", count=count)
        if kind == "string":   # fixed-length strings
            n = dtype[1]
            return [raw[k * n:(k + 1) * n].split(b"\0")[0].decode("utf-8") for k in range(count)]
        if kind == "compound":
            names = [m[0] for m in dtype[2]]
            if names in (["re", "im"], ["re_", "im_"]):
                a = np.frombuffer(raw, dtype="<f8", count=2 * count).reshape(count, 2)
                return a[:, 0] + 1j * a[:, 1]
            size = dtype[1]
            recs = []
            for k in range(count):
                rec = {}
                for (name, moff, mt, msz) in dtype[2]:
                    rec[name] = self._decode(mt, raw[k * size + moff:k * size + moff + msz], 1)[0]
                recs.append(rec)
            return recs
        raise NotImplementedError(kind)

    def read(self, addr):
        dims, dtype, raw = self.dataset(addr)
        count = int(np.prod(dims)) if dims else 1
        vals = self._decode(dtype, raw, count)
        if dtype[0] == "compound" and isinstance(vals, list):
            rec = vals[0]
            rec = {k.rstrip("_"): v for k, v in rec.items()}
            if set(rec) >= {"m", "n", "colptr", "rowval", "nzval"}:
                colptr = np.asarray(self.read(int(rec["colptr"])), dtype=np.int64)
                rowval = np.asarray(self.read(int(rec["rowval"])), dtype=np.int64)
                nzval = np.asarray(self.read(int(rec["nzval"])))
                return sps.csc_matrix((nzval, rowval - 1, colptr - 1),
                                      shape=(int(rec["m"]), int(rec["n"])))
            return vals if len(vals) > 1 else rec
        if not dims:
            return vals[0]
        # HDF5 stores row-major with Julia dims reversed -> column-major view
        return np.asarray(vals).reshape(dims[::-1], order="F") if len(dims) > 1 else np.asarray(vals)


def load_tree(path):
    """Every dataset of an HDF5/JLD file as {"group/.../name": value}, groups
    walked recursively (JLD's `_types` and `_refs` included)."""
    r = _Reader(path)
    out = {}

    def is_group(addr):
        return any(mtype in (0x02, 0x06, 0x11) for mtype, _, _ in r.messages(addr))

    def walk(addr, prefix):
        for name, a in r.links(addr).items():
            full = f"{prefix}{name}"
            if is_group(a):
                walk(a, full + "/")
            else:
                out[full] = r.read(a)

    walk(r.root, "")
    return out


def load_jld(path):
    """Return {name: value} for every top-level dataset of a JLD file."""
    r = _Reader(path)
    out = {}
    for name, addr in r.links(r.root).items():
        if name.startswith("_"):
            continue
        try:
            out[name] = r.read(addr)
        except Exception as exc:     # pragma: no cover - reported by the caller
            out[name] = exc
    return out
