"""Minimal read-only HDF5 reader, written from the public HDF5 file-format specification.

It covers exactly what the reference's small test fixtures use: a version-0 superblock,
symbol-table groups (v1 B-trees 'TREE', local heaps 'HEAP', symbol nodes 'SNOD'),
version-1 object headers (with continuation blocks), and contiguous or compact datasets
of IEEE floats / integers, or compound {r, i} float pairs (how HDF5.jl stores complex
numbers).  No h5py / libhdf5 is available, and nothing else is needed for the fixtures.
"""
from __future__ import annotations

import struct
from typing import Dict

import numpy as np

SIG = b"\x89HDF\r\n\x1a\n"


class H5File:
    def __init__(self, path: str):
        with open(path, "rb") as f:
            self.buf = f.read()
        b = self.buf
        if b[:8] != SIG:
            raise ValueError("not an HDF5 file")
        if b[8] != 0:
            raise NotImplementedError(f"superblock version {b[8]}")
        self.so = b[13]   # size of offsets
        self.sl = b[14]   # size of lengths
        pos = 8 + 16
        pos += 4 * self.so  # base, free-space, eof, driver
        self.root = self._symbol_entry(pos)

    # -- primitive readers ---------------------------------------------------
    def _u(self, pos, n):
        return int.from_bytes(self.buf[pos:pos + n], "little")

    def _symbol_entry(self, pos):
        so = self.so
        name_off = self._u(pos, so)
        ohdr = self._u(pos + so, so)
        cache = self._u(pos + 2 * so, 4)
        scratch = pos + 2 * so + 8
        btree = heap = None
        if cache == 1:
            btree = self._u(scratch, so)
            heap = self._u(scratch + so, so)
        return dict(name_off=name_off, ohdr=ohdr, btree=btree, heap=heap)

    def _heap_data(self, addr):
        b = self.buf
        assert b[addr:addr + 4] == b"HEAP"
        so, sl = self.so, self.sl
        data_addr = self._u(addr + 8 + 2 * sl, so)
        return data_addr

    def _heap_name(self, heap_data, off):
        end = self.buf.index(b"\x00", heap_data + off)
        return self.buf[heap_data + off:end].decode()

    def _group_entries(self, btree, heap):
        heap_data = self._heap_data(heap)
        out = {}
        self._walk_btree(btree, heap_data, out)
        return out

    def _walk_btree(self, addr, heap_data, out):
        b = self.buf
        so, sl = self.so, self.sl
        assert b[addr:addr + 4] == b"TREE", "bad B-tree node"
        level = b[addr + 5]
        n = self._u(addr + 6, 2)
        pos = addr + 8 + 2 * so
        pos += sl  # key 0
        for _ in range(n):
            child = self._u(pos, so)
            pos += so + sl
            if level > 0:
                self._walk_btree(child, heap_data, out)
            else:
                self._read_snod(child, heap_data, out)

    def _read_snod(self, addr, heap_data, out):
        b = self.buf
        assert b[addr:addr + 4] == b"SNOD"
        n = self._u(addr + 6, 2)
        pos = addr + 8
        esz = 2 * self.so + 24
        for i in range(n):
            e = self._symbol_entry(pos + i * esz)
            out[self._heap_name(heap_data, e["name_off"])] = e

    def _messages(self, addr):
        b = self.buf
        if b[addr] != 1:
            raise NotImplementedError("only version-1 object headers")
        nmsg = self._u(addr + 2, 2)
        size = self._u(addr + 8, 4)
        blocks = [(addr + 16, size)]
        msgs = []
        while blocks and len(msgs) < nmsg:
            start, length = blocks.pop(0)
            pos = start
            while pos + 8 <= start + length and len(msgs) < nmsg:
                mtype = self._u(pos, 2)
                msize = self._u(pos + 2, 2)
                data = pos + 8
                if mtype == 0x10:  # continuation
                    blocks.append((self._u(data, self.so), self._u(data + self.so, self.sl)))
                msgs.append((mtype, data, msize))
                pos = data + msize
        return msgs

    # -- public API ----------------------------------------------------------
    def _links(self, ohdr):
        """Children of a group: link messages (new-style) or the symbol table (old-style)."""
        links = {}
        symtab = None
        for mtype, data, _ in self._messages(ohdr):
            if mtype == 0x06:
                name, addr = self._link_message(data)
                links[name] = dict(name_off=None, ohdr=addr, btree=None, heap=None)
            elif mtype == 0x11:
                symtab = (self._u(data, self.so), self._u(data + self.so, self.so))
        if links:
            return links
        if symtab is not None:
            return self._group_entries(*symtab)
        return {}

    def _link_message(self, pos):
        b = self.buf
        flags = b[pos + 1]
        p = pos + 2
        ltype = 0
        if flags & 0x08:
            ltype = b[p]; p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nlen_size = 1 << (flags & 0x03)
        nlen = self._u(p, nlen_size); p += nlen_size
        name = b[p:p + nlen].decode(); p += nlen
        if ltype != 0:
            raise NotImplementedError("soft/external links")
        return name, self._u(p, self.so)

    def _resolve(self, path: str):
        ent = self.root
        for part in [p for p in path.split("/") if p]:
            ent = self._links(ent["ohdr"])[part]
        return ent

    def list(self, path: str = "/") -> Dict[str, dict]:
        return self._links(self._resolve(path)["ohdr"])

    def read(self, path: str) -> np.ndarray:
        ent = self._resolve(path)
        shape = dtype = layout = None
        for mtype, data, msize in self._messages(ent["ohdr"]):
            if mtype == 0x01:
                shape = self._dataspace(data)
            elif mtype == 0x03:
                dtype = self._datatype(data)
            elif mtype == 0x08:
                layout = self._layout(data)
        if shape is None or dtype is None or layout is None:
            raise ValueError(f"{path}: not a dataset")
        count = int(np.prod(shape)) if shape else 1
        kind, addr, nbytes = layout
        raw = self.buf[addr:addr + count * dtype.itemsize]
        arr = np.frombuffer(raw, dtype=dtype, count=count)
        if dtype.names == ("r", "i"):
            arr = arr["r"] + 1j * arr["i"]
        # HDF5 stores C order of the reversed Julia dims: reshape then reverse axes.
        arr = arr.reshape(shape)
        return np.ascontiguousarray(np.transpose(arr)) if arr.ndim > 1 else arr.copy()

    def _dataspace(self, pos):
        b = self.buf
        version = b[pos]
        ndims = b[pos + 1]
        if version == 1:
            p = pos + 8
        elif version == 2:
            p = pos + 4
        else:
            raise NotImplementedError(f"dataspace v{version}")
        return tuple(self._u(p + i * self.sl, self.sl) for i in range(ndims))

    def _datatype(self, pos):
        b = self.buf
        cls = b[pos] & 0x0F
        version = b[pos] >> 4
        size = self._u(pos + 4, 4)
        if cls == 1:   # floating point
            return np.dtype("<f%d" % size)
        if cls == 0:   # fixed point
            signed = (b[pos + 1] >> 3) & 1
            return np.dtype(("<i%d" if signed else "<u%d") % size)
        if cls == 6:   # compound
            nmem = self._u(pos + 1, 2)
            p = pos + 8
            fields = []
            for _ in range(nmem):
                end = b.index(b"\x00", p)
                name = b[p:end].decode()
                if version < 3:
                    namelen = ((end - p) // 8 + 1) * 8
                    p += namelen
                    off = self._u(p, 4)
                    p += 4 + 1 + 3 + 4 + 4 + 16
                else:
                    p = end + 1
                    nb = max(1, (size.bit_length() + 7) // 8)
                    off = self._u(p, nb)
                    p += nb
                sub = self._datatype(p)
                p += 8 + self._props_len(p)
                fields.append((name, off, sub))
            return np.dtype({"names": [f[0] for f in fields], "formats": [f[2] for f in fields],
                             "offsets": [f[1] for f in fields], "itemsize": size})
        raise NotImplementedError(f"datatype class {cls}")

    def _props_len(self, pos):
        cls = self.buf[pos] & 0x0F
        if cls == 1:
            return 12
        if cls == 0:
            return 4
        raise NotImplementedError("nested compound")

    def _layout(self, pos):
        b = self.buf
        version = b[pos]
        if version == 3:
            cls = b[pos + 1]
            if cls == 1:   # contiguous
                return ("contiguous", self._u(pos + 2, self.so), self._u(pos + 2 + self.so, self.sl))
            if cls == 0:   # compact
                n = self._u(pos + 2, 2)
                return ("compact", pos + 4, n)
            raise NotImplementedError("chunked layout")
        if version in (1, 2):
            ndims = b[pos + 1]
            cls = b[pos + 2]
            p = pos + 8
            addr = self._u(p, self.so)
            if cls == 1:
                return ("contiguous", addr, None)
            if cls == 0:
                p += ndims * 4
                n = self._u(p, 4)
                return ("compact", p + 4, n)
            raise NotImplementedError("chunked layout")
        raise NotImplementedError(f"layout v{version}")
