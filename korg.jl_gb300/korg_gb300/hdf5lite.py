"""Minimal read-only HDF5 reader for the classic (superblock v0) files Korg ships.

Korg's data tables (the Stehle & Hutcheon hydrogen Stark profiles, the atomic partition
functions, the Lyman golden vector used by its tests) are HDF5 files written by HDF5.jl with
the classic layout: superblock version 0, version-1 object headers, groups stored as symbol
tables (v1 B-trees + local heaps), contiguous or compact datasets and attributes of fixed-size
numeric types.  This module reads exactly that subset (plus fixed and variable length strings
well enough to read attribute names) and raises ``NotImplementedError`` on anything else, so
no h5py / libhdf5 is needed on either machine.

Arrays are returned in the file's (C / row-major) dimension order.  Julia's ``read`` returns
the same data with the dimension order reversed (column-major), so a Julia array of size
``(nT, nNe, nD)`` arrives here with shape ``(nD, nNe, nT)``.
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np

_SIG = b"\x89HDF\r\n\x1a\n"
_UNDEF = 0xFFFFFFFFFFFFFFFF


@dataclass
class _Datatype:
    cls: int
    size: int
    dtype: np.dtype | None  # None for strings / unsupported


@dataclass
class Node:
    """A group or dataset.  ``children`` is filled for groups, ``attrs`` for both."""

    name: str
    kind: str  # "group" | "dataset"
    attrs: dict = field(default_factory=dict)
    children: dict = field(default_factory=dict)
    _shape: tuple | None = None
    _dtype: _Datatype | None = None
    _layout: tuple | None = None  # ("contiguous", addr, size) | ("compact", bytes)

    def __getitem__(self, key):
        node = self
        for part in [p for p in key.split("/") if p]:
            node = node.children[part]
        return node

    def keys(self):
        return list(self.children.keys())


class File:
    """Parse the whole object tree of an HDF5 file on open (the files are small)."""

    def __init__(self, path):
        with open(path, "rb") as f:
            self.buf = f.read()
        b = self.buf
        if b[:8] != _SIG:
            raise ValueError(f"{path}: not an HDF5 file")
        if b[8] != 0:
            raise NotImplementedError(f"superblock version {b[8]}")
        self.so, self.sl = b[13], b[14]
        if self.so != 8 or self.sl != 8:
            raise NotImplementedError("only 8-byte offsets/lengths are supported")
        # root group symbol table entry follows the 4 addresses at offset 24
        ent = 24 + 4 * 8
        hdr_addr = self._u64(ent + 8)
        self.root = self._read_object("/", hdr_addr)

    # ------------------------------------------------------------------ primitives
    def _u64(self, off):
        return struct.unpack_from("<Q", self.buf, off)[0]

    def _cstr(self, off):
        end = self.buf.index(b"\x00", off)
        return self.buf[off:end].decode()

    # ------------------------------------------------------------------ objects
    def _messages(self, addr):
        b = self.buf
        version = b[addr]
        if version != 1:
            raise NotImplementedError(f"object header version {version}")
        nmsg = struct.unpack_from("<H", b, addr + 2)[0]
        hsize = struct.unpack_from("<I", b, addr + 8)[0]
        blocks = [(addr + 16, hsize)]
        out = []
        while blocks and len(out) < nmsg:
            start, size = blocks.pop(0)
            p = start
            while p + 8 <= start + size and len(out) < nmsg:
                mtype, msize, mflags = struct.unpack_from("<HHB", b, p)
                data = b[p + 8:p + 8 + msize]
                p += 8 + msize
                if mtype == 0x10:  # continuation
                    blocks.append(struct.unpack_from("<QQ", data, 0))
                out.append((mtype, data, mflags))
        return out

    def _read_object(self, name, addr):
        msgs = self._messages(addr)
        node = Node(name=name, kind="dataset")
        is_group = False
        for mtype, data, _ in msgs:
            if mtype == 0x11:  # symbol table -> group
                is_group = True
                btree, heap = struct.unpack_from("<QQ", data, 0)
                for cname, caddr in self._group_entries(btree, heap):
                    node.children[cname] = self._read_object(cname, caddr)
            elif mtype == 0x06:  # link message (compact "new style" group)
                is_group = True
                link = self._link(data)
                if link is not None:
                    node.children[link[0]] = self._read_object(link[0], link[1])
            elif mtype == 0x02:  # link info: links may live in a fractal heap (dense storage)
                is_group = True
                fheap = struct.unpack_from("<Q", data, 2 + (8 if data[1] & 1 else 0))[0]
                if fheap != _UNDEF:
                    for cname, caddr in self._dense_links(fheap):
                        node.children[cname] = self._read_object(cname, caddr)
            elif mtype == 0x01:
                node._shape = self._dataspace(data)
            elif mtype == 0x03:
                node._dtype = self._datatype(data)
            elif mtype == 0x08:
                node._layout = self._layout_msg(data)
            elif mtype == 0x0C:
                aname, aval = self._attribute(data)
                node.attrs[aname] = aval
        node.kind = "group" if is_group else "dataset"
        return node

    def _group_entries(self, btree_addr, heap_addr):
        b = self.buf
        if b[heap_addr:heap_addr + 4] != b"HEAP":
            raise ValueError("bad local heap")
        heap_data = self._u64(heap_addr + 24)
        entries = []

        def walk(addr):
            if b[addr:addr + 4] != b"TREE":
                raise ValueError("bad v1 B-tree node")
            ntype, level = b[addr + 4], b[addr + 5]
            used = struct.unpack_from("<H", b, addr + 6)[0]
            if ntype != 0:
                raise NotImplementedError("chunked-data B-trees are not supported")
            p = addr + 24  # after signature, type, level, used, 2 sibling addresses
            p += 8  # key 0
            for _ in range(used):
                child = self._u64(p)
                p += 16  # child + next key
                if level > 0:
                    walk(child)
                else:
                    snod(child)

        def snod(addr):
            if b[addr:addr + 4] != b"SNOD":
                raise ValueError("bad symbol table node")
            nsym = struct.unpack_from("<H", b, addr + 6)[0]
            p = addr + 8
            for _ in range(nsym):
                name_off, hdr = struct.unpack_from("<QQ", b, p)
                entries.append((self._cstr(heap_data + name_off), hdr))
                p += 40

        walk(btree_addr)
        return entries

    def _dense_links(self, fheap_addr):
        """Links of a dense-storage group: walk the fractal heap's managed direct blocks from
        its root block and decode the link messages packed in each (unfiltered heaps only)."""
        b = self.buf
        if b[fheap_addr:fheap_addr + 4] != b"FRHP":
            raise ValueError("bad fractal heap header")
        p = fheap_addr + 5
        heap_id_len, filt_len = struct.unpack_from("<HH", b, p)
        flags = b[p + 4]
        if filt_len:
            raise NotImplementedError("filtered fractal heaps")
        p += 5 + 4 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8 + 8
        width = struct.unpack_from("<H", b, p)[0]
        start_size, max_direct = struct.unpack_from("<QQ", b, p + 2)
        max_heap_bits, _start_rows = struct.unpack_from("<HH", b, p + 18)
        root, cur_rows = struct.unpack_from("<QH", b, p + 22)
        off_bytes = (max_heap_bits + 7) // 8
        dblock_hdr = 4 + 1 + 8 + off_bytes + (4 if flags & 0x02 else 0)

        def row_size(r):
            return start_size if r < 2 else start_size * (1 << (r - 1))

        blocks = []

        def indirect(addr, nrows):
            if b[addr:addr + 4] != b"FHIB":
                raise ValueError("bad fractal heap indirect block")
            q = addr + 4 + 1 + 8 + off_bytes
            for r in range(nrows):
                for _ in range(width):
                    child = struct.unpack_from("<Q", b, q)[0]
                    q += 8
                    if child == _UNDEF:
                        continue
                    size = row_size(r)
                    if size <= max_direct:
                        blocks.append((child, size))
                    else:
                        raise NotImplementedError("nested fractal heap indirect blocks")

        if cur_rows == 0:
            blocks.append((root, start_size))
        else:
            indirect(root, cur_rows)
        links = []
        for addr, size in blocks:
            if b[addr:addr + 4] != b"FHDB":
                raise ValueError("bad fractal heap direct block")
            q, end = addr + dblock_hdr, addr + size
            while q < end and b[q] == 1:  # link message version 1
                name, caddr, used = self._link_len(b[q:end])
                links.append((name, caddr))
                q += used
        return links

    @staticmethod
    def _link_len(data):
        flags = data[1]
        p = 2
        if flags & 0x08:
            if data[p] != 0:
                raise NotImplementedError("non-hard links in dense storage")
            p += 1
        if flags & 0x04:
            p += 8
        if flags & 0x10:
            p += 1
        nlen_size = 1 << (flags & 0x03)
        nlen = int.from_bytes(data[p:p + nlen_size], "little")
        p += nlen_size
        name = bytes(data[p:p + nlen]).decode()
        p += nlen
        return name, struct.unpack_from("<Q", data, p)[0], p + 8

    @staticmethod
    def _link(data):
        """Decode a version-1 link message; returns (name, object header address) or None."""
        flags = data[1]
        p = 2
        ltype = 0
        if flags & 0x08:
            ltype = data[p]
            p += 1
        if flags & 0x04:
            p += 8  # creation order
        if flags & 0x10:
            p += 1  # character set
        nlen_size = 1 << (flags & 0x03)
        nlen = int.from_bytes(data[p:p + nlen_size], "little")
        p += nlen_size
        name = bytes(data[p:p + nlen]).decode()
        p += nlen
        if ltype != 0:  # soft / external links are not followed
            return None
        return name, struct.unpack_from("<Q", data, p)[0]

    @staticmethod
    def _dataspace(data):
        version, ndims, flags = data[0], data[1], data[2]
        if version == 1:
            p = 8
        elif version == 2:
            p = 4
            if data[3] == 0:  # scalar
                return ()
            if data[3] == 2:  # null
                return None
        else:
            raise NotImplementedError(f"dataspace version {version}")
        return tuple(struct.unpack_from("<Q", data, p + 8 * i)[0] for i in range(ndims))

    @staticmethod
    def _datatype(data):
        cls = data[0] & 0x0F
        bits = data[1] | (data[2] << 8) | (data[3] << 16)
        size = struct.unpack_from("<I", data, 4)[0]
        order = ">" if (bits & 1) else "<"
        if cls == 0:  # fixed point
            signed = bool(bits & 0x08)
            return _Datatype(cls, size, np.dtype(f"{order}{'i' if signed else 'u'}{size}"))
        if cls == 1:  # floating point
            return _Datatype(cls, size, np.dtype(f"{order}f{size}"))
        return _Datatype(cls, size, None)

    @staticmethod
    def _layout_msg(data):
        version = data[0]
        if version != 3:
            raise NotImplementedError(f"data layout version {version}")
        lclass = data[1]
        if lclass == 0:
            size = struct.unpack_from("<H", data, 2)[0]
            return ("compact", bytes(data[4:4 + size]))
        if lclass == 1:
            addr, size = struct.unpack_from("<QQ", data, 2)
            return ("contiguous", addr, size)
        raise NotImplementedError("chunked datasets are not supported")

    def _attribute(self, data):
        version = data[0]
        nsz, tsz, ssz = struct.unpack_from("<HHH", data, 2)
        if version == 1:
            pad = lambda n: (n + 7) // 8 * 8
            p = 8
        elif version in (2, 3):
            pad = lambda n: n
            p = 8 if version == 2 else 9  # v3 adds a name-encoding byte
        else:
            raise NotImplementedError(f"attribute message version {version}")
        name = bytes(data[p:p + nsz]).split(b"\x00")[0].decode()
        p += pad(nsz)
        dt = self._datatype(data[p:p + tsz])
        p += pad(tsz)
        shape = self._dataspace(data[p:p + ssz])
        p += pad(ssz)
        raw = bytes(data[p:])
        if dt.dtype is None:
            if dt.cls == 3:  # fixed-length string
                return name, raw[:dt.size].split(b"\x00")[0].decode()
            return name, None  # variable-length and other classes are not decoded
        n = int(np.prod(shape)) if shape else 1
        arr = np.frombuffer(raw[:n * dt.size], dtype=dt.dtype).astype(dt.dtype.newbyteorder("="))
        if not shape:
            return name, arr[0].item()
        return name, arr.reshape(shape)

    # ------------------------------------------------------------------ public
    def read(self, path):
        node = self.root[path]
        if node.kind != "dataset":
            raise ValueError(f"{path} is a group")
        dt, shape, layout = node._dtype, node._shape, node._layout
        if dt is None or (dt.dtype is None and dt.cls not in (3, 9)):
            raise NotImplementedError(f"{path}: unsupported datatype")
        n = int(np.prod(shape)) if shape else 1
        if layout[0] == "contiguous":
            addr, size = layout[1], layout[2]
            if addr == _UNDEF:
                raw = b"\x00" * (n * dt.size)
            else:
                raw = self.buf[addr:addr + n * dt.size]
        else:
            raw = layout[1][:n * dt.size]
        if dt.cls == 3:  # fixed-length strings, NUL padded
            vals = [raw[i * dt.size:(i + 1) * dt.size].split(b"\x00")[0].decode() for i in range(n)]
        elif dt.cls == 9:  # variable-length strings: (length, global heap address, object index)
            vals = [self._global_heap_object(*struct.unpack_from("<IQI", raw, 16 * i)) for i in range(n)]
        else:
            arr = np.frombuffer(raw, dtype=dt.dtype).astype(dt.dtype.newbyteorder("="))
            return arr.reshape(shape) if shape else arr[0].item()
        return np.array(vals, dtype=object).reshape(shape) if shape else vals[0]

    def _global_heap_object(self, length, collection, index):
        """The bytes of object ``index`` of a global heap collection ("GCOL"), decoded as text."""
        b = self.buf
        if b[collection:collection + 4] != b"GCOL":
            raise ValueError("bad global heap collection")
        end = collection + self._u64(collection + 8)
        p = collection + 16
        while p + 16 <= end:
            idx = struct.unpack_from("<H", b, p)[0]
            size = self._u64(p + 8)
            if idx == 0:  # free space ends the collection
                break
            if idx == index:
                return b[p + 16:p + 16 + min(size, length)].decode()
            p += 16 + (size + 7) // 8 * 8
        raise ValueError(f"global heap object {index} not found")

    def __getitem__(self, path):
        return self.root[path]

    def keys(self):
        return self.root.keys()
