"""A minimal HDF5 reader for the tests (test infrastructure only, not part of the product).

It reads the subset of the HDF5 file format (format specification 1.x/2.0, superblock version 0)
that classic libhdf5 writes by default and that the output writer in this project produces:

* superblock version 0 (8-byte offsets and lengths, optional user block before it);
* groups as symbol tables: a version-1 B-tree of group nodes (type 0) over symbol-table nodes
  ("SNOD") whose names live in a local heap ("HEAP");
* version-1 object headers with continuation blocks;
* messages: NIL (0x0), dataspace (0x1), datatype (0x3), fill value (0x4/0x5), data layout (0x8,
  versions 1-3, compact and contiguous), attribute (0xC, listed by name only), continuation
  (0x10), symbol table (0x11), modification time (0x12/0xE).

It checks every signature, version and count that it reads, so a malformed file raises
``H5FormatError`` instead of returning data.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Tuple

import numpy as np

UNDEF = 0xFFFFFFFFFFFFFFFF
SIGNATURE = b"\x89HDF\r\n\x1a\n"


class H5FormatError(ValueError):
    pass


@dataclass
class Message:
    type: int
    flags: int
    body: bytes


@dataclass
class Dataset:
    name: str
    shape: Tuple[int, ...]
    dtype: np.dtype
    layout: str
    address: int
    size: int
    data: np.ndarray
    messages: List[int] = field(default_factory=list)
    attributes: List[str] = field(default_factory=list)


@dataclass
class Group:
    name: str
    members: Dict[str, object] = field(default_factory=dict)
    messages: List[int] = field(default_factory=list)


class File:
    """Parses the whole file at construction: ``root`` is a Group tree of Groups and Datasets."""

    def __init__(self, path: str):
        with open(path, "rb") as fh:
            self.buf = fh.read()
        self.base = self._find_superblock()
        self._parse_superblock()
        self.root = self._read_group("/", self.root_ohdr)

    # ------------------------------------------------------------------ primitives
    def _u(self, fmt: str, off: int):
        try:
            return struct.unpack_from("<" + fmt, self.buf, off)
        except struct.error as e:
            raise H5FormatError(f"read past the end of the file at {off}") from e

    def _abs(self, addr: int) -> int:
        if addr == UNDEF:
            raise H5FormatError("undefined address where one is required")
        a = self.base + addr
        if a >= len(self.buf):
            raise H5FormatError(f"address {addr} beyond the end of the file")
        return a

    def _find_superblock(self) -> int:
        off = 0
        while off < len(self.buf):
            if self.buf[off:off + 8] == SIGNATURE:
                return off
            off = 512 if off == 0 else off * 2
        raise H5FormatError("no HDF5 signature at 0, 512, 1024, ...")

    def _parse_superblock(self) -> None:
        o = self.base + 8
        ver, fs_ver, root_ver, _r, sh_ver, so, sl, _r2 = self._u("8B", o)
        if ver != 0 or fs_ver != 0 or root_ver != 0 or sh_ver != 0:
            raise H5FormatError(f"superblock version {ver} (only version 0 is read)")
        if so != 8 or sl != 8:
            raise H5FormatError("only 8-byte offsets and lengths are read")
        self.leaf_k, self.internal_k, self.flags = self._u("HHI", o + 8)
        if self.leaf_k == 0 or self.internal_k == 0:
            raise H5FormatError("group K values must be > 0")
        base_addr, fs_addr, self.eof, drv = self._u("4Q", o + 16)
        if base_addr != self.base:
            raise H5FormatError(f"base address {base_addr} does not match the superblock offset {self.base}")
        if drv != UNDEF:
            raise H5FormatError("driver information block not supported")
        # libhdf5 stores the end-of-file address including any user block
        if self.eof > len(self.buf):
            raise H5FormatError(f"end-of-file address {self.eof} beyond the file size")
        _name, self.root_ohdr, cache, _res = self._u("QQII", o + 48)
        self.root_cache = cache
        self.root_scratch = self._u("QQ", o + 72) if cache == 1 else None

    # ------------------------------------------------------------------ object headers
    def _messages(self, addr: int) -> List[Message]:
        a = self._abs(addr)
        ver, _r, nmsg, refc, size = self._u("BBHII", a)
        if ver != 1:
            raise H5FormatError(f"object header version {ver} at {addr} (only version 1 is read)")
        blocks = [(a + 16, size)]
        out: List[Message] = []
        while blocks:
            start, length = blocks.pop(0)
            p, end = start, start + length
            while p < end:
                if end - p < 8:
                    raise H5FormatError("truncated message header")
                mtype, msize, mflags = self._u("HHB", p)
                if msize % 8:
                    raise H5FormatError(f"message size {msize} not a multiple of 8")
                body = self.buf[p + 8:p + 8 + msize]
                if len(body) != msize or p + 8 + msize > end:
                    raise H5FormatError("message runs past its header block")
                out.append(Message(mtype, mflags, body))
                if mtype == 0x10:
                    caddr, clen = struct.unpack_from("<QQ", body)
                    blocks.append((self._abs(caddr), clen))
                p += 8 + msize
        if len(out) != nmsg:
            raise H5FormatError(f"object header at {addr}: {len(out)} messages, header says {nmsg}")
        if refc < 1:
            raise H5FormatError("object reference count < 1")
        return out

    # ------------------------------------------------------------------ groups
    def _heap(self, addr: int) -> Tuple[bytes, int]:
        a = self._abs(addr)
        if self.buf[a:a + 4] != b"HEAP":
            raise H5FormatError("local heap signature")
        if self.buf[a + 4] != 0:
            raise H5FormatError("local heap version")
        dsize, free, daddr = self._u("QQQ", a + 8)
        if free != 1 and free != UNDEF and free >= dsize:
            raise H5FormatError("bad local heap free list")
        d = self._abs(daddr)
        data = self.buf[d:d + dsize]
        if len(data) != dsize:
            raise H5FormatError("local heap data segment past the end of the file")
        if data[:1] != b"\x00":
            raise H5FormatError("local heap offset 0 must hold the empty string")
        return data, dsize

    @staticmethod
    def _heap_str(heap: bytes, off: int) -> str:
        e = heap.find(b"\x00", off)
        if off >= len(heap) or e < 0:
            raise H5FormatError("name offset outside the local heap")
        return heap[off:e].decode()

    def _btree_leaves(self, addr: int, heap: bytes) -> List[int]:
        a = self._abs(addr)
        if self.buf[a:a + 4] != b"TREE":
            raise H5FormatError("B-tree signature")
        ntype, level, used = self._u("BBH", a + 4)
        if ntype != 0:
            raise H5FormatError("group B-tree node type must be 0")
        if used > 2 * self.internal_k:
            raise H5FormatError("B-tree node has more children than 2K")
        p = a + 24
        keys, children = [], []
        for i in range(used):
            keys.append(self._u("Q", p)[0])
            children.append(self._u("Q", p + 8)[0])
            p += 16
        keys.append(self._u("Q", p)[0])
        names = [self._heap_str(heap, k) for k in keys]
        for i in range(1, len(names)):
            if names[i - 1] > names[i]:
                raise H5FormatError("B-tree keys out of order")
        if level == 0:
            return children
        out: List[int] = []
        for c in children:
            out += self._btree_leaves(c, heap)
        return out

    def _read_group(self, name: str, ohdr: int) -> Group:
        msgs = self._messages(ohdr)
        stab = [m for m in msgs if m.type == 0x11]
        if len(stab) != 1:
            raise H5FormatError(f"group {name}: expected one symbol table message")
        bt, hp = struct.unpack_from("<QQ", stab[0].body)
        heap, _ = self._heap(hp)
        g = Group(name, messages=[m.type for m in msgs])
        last = None
        for snod in self._btree_leaves(bt, heap):
            a = self._abs(snod)
            if self.buf[a:a + 4] != b"SNOD" or self.buf[a + 4] != 1:
                raise H5FormatError("symbol table node signature/version")
            (nsym,) = self._u("H", a + 6)
            if nsym > 2 * self.leaf_k:
                raise H5FormatError("symbol table node holds more than 2K entries")
            for e in range(nsym):
                p = a + 8 + 40 * e
                noff, oaddr, cache, _r = self._u("QQII", p)
                mname = self._heap_str(heap, noff)
                if last is not None and mname <= last:
                    raise H5FormatError(f"group {name}: names not in strictly increasing order")
                last = mname
                full = name.rstrip("/") + "/" + mname
                sub = self._messages(oaddr)
                if any(m.type == 0x11 for m in sub):
                    if cache == 1:
                        sbt, shp = self._u("QQ", p + 24)
                        own = [m for m in sub if m.type == 0x11][0]
                        if (sbt, shp) != struct.unpack_from("<QQ", own.body):
                            raise H5FormatError(f"{full}: cached scratch-pad differs from the symbol table message")
                    g.members[mname] = self._read_group(full, oaddr)
                else:
                    g.members[mname] = self._read_dataset(full, sub)
        return g

    # ------------------------------------------------------------------ datasets
    @staticmethod
    def _dataspace(body: bytes) -> Tuple[int, ...]:
        ver, rank, flags = struct.unpack_from("<BBB", body)
        if ver == 1:
            off = 8
        elif ver == 2:
            off = 4
        else:
            raise H5FormatError(f"dataspace version {ver}")
        dims = struct.unpack_from("<" + "Q" * rank, body, off)
        return tuple(int(d) for d in dims)

    @staticmethod
    def _datatype(body: bytes) -> np.dtype:
        cv = body[0]
        cls, ver = cv & 0x0F, cv >> 4
        if ver not in (1, 2, 3):
            raise H5FormatError(f"datatype version {ver}")
        bits0 = body[1]
        (size,) = struct.unpack_from("<I", body, 4)
        order = ">" if bits0 & 1 else "<"
        if cls == 1:  # floating point
            off, prec, eloc, esize, mloc, msize, bias = struct.unpack_from("<HHBBBBI", body, 8)
            known = {(8, 64, 52, 11, 0, 52, 1023): "f8", (4, 32, 23, 8, 0, 23, 127): "f4"}
            key = (size, prec, eloc, esize, mloc, msize, bias)
            if off != 0 or key not in known:
                raise H5FormatError(f"unsupported floating-point layout {key}")
            if (bits0 >> 4) & 3 != 2:
                raise H5FormatError("mantissa normalisation must be 'implied msb'")
            return np.dtype(order + known[key])
        if cls == 0:  # fixed point
            signed = bool(bits0 & 8)
            return np.dtype(order + ("i" if signed else "u") + str(size))
        raise H5FormatError(f"datatype class {cls} not supported")

    def _read_dataset(self, name: str, msgs: List[Message]) -> Dataset:
        by = {}
        for m in msgs:
            by.setdefault(m.type, []).append(m)
        for req in (0x1, 0x3, 0x8):
            if len(by.get(req, [])) != 1:
                raise H5FormatError(f"dataset {name}: message 0x{req:x} missing or repeated")
        shape = self._dataspace(by[0x1][0].body)
        dt = self._datatype(by[0x3][0].body)
        lay = by[0x8][0].body
        lver = lay[0]
        if lver == 3:
            lcls = lay[1]
            if lcls == 1:
                addr, size = struct.unpack_from("<QQ", lay, 2)
                layout = "contiguous"
                n = int(np.prod(shape)) if shape else 1
                if size != n * dt.itemsize:
                    raise H5FormatError(f"dataset {name}: layout size {size} != {n} x {dt.itemsize}")
                a = self._abs(addr) if n else 0
                raw = self.buf[a:a + size]
            elif lcls == 0:
                (size,) = struct.unpack_from("<H", lay, 2)
                raw = lay[4:4 + size]
                addr, layout = UNDEF, "compact"
            else:
                raise H5FormatError(f"dataset {name}: layout class {lcls} (chunked) not supported")
        elif lver in (1, 2):
            rank, lcls = lay[1], lay[2]
            if lcls != 1:
                raise H5FormatError(f"dataset {name}: layout class {lcls} not supported")
            (addr,) = struct.unpack_from("<Q", lay, 8)
            layout = "contiguous"
            n = int(np.prod(shape)) if shape else 1
            size = n * dt.itemsize
            a = self._abs(addr)
            raw = self.buf[a:a + size]
        else:
            raise H5FormatError(f"layout version {lver}")
        if len(raw) != size:
            raise H5FormatError(f"dataset {name}: raw data past the end of the file")
        data = np.frombuffer(raw, dtype=dt).reshape(shape)
        attrs = []
        for m in by.get(0xC, []):
            ver = m.body[0]
            (nlen,) = struct.unpack_from("<H", m.body, 2)
            if ver == 1:
                attrs.append(m.body[8:8 + nlen].rstrip(b"\x00").decode())
        return Dataset(name, shape, dt, layout, addr, size, data.copy(), [m.type for m in msgs], attrs)

    # ------------------------------------------------------------------ access
    def __getitem__(self, path: str):
        node = self.root
        for part in [p for p in path.split("/") if p]:
            if not isinstance(node, Group) or part not in node.members:
                raise KeyError(path)
            node = node.members[part]
        return node

    def datasets(self) -> Dict[str, Dataset]:
        out: Dict[str, Dataset] = {}

        def walk(g: Group):
            for m in g.members.values():
                if isinstance(m, Group):
                    walk(m)
                else:
                    out[m.name] = m

        walk(self.root)
        return out
