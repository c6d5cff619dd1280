"""A minimal read-only HDF5 reader, for files written by h5py with its
default (earliest) format: superblock version 0, version-1 object headers,
groups stored as symbol tables (version-1 B-trees of symbol-table nodes plus
a local heap of link names), datasets with contiguous or compact layout and
integer or IEEE floating-point elements.  Chunked / compressed datasets and
newer structures raise ValueError.

Written from the published HDF5 file-format specification (superblock,
"TREE"/"SNOD"/"HEAP" structures, object header messages 0x0001 dataspace,
0x0003 datatype, 0x0008 data layout, 0x0010 continuation, 0x0011 symbol
table).  It lets fastpli_gb300.io load .h5 fiber-bundle files without h5py,
and the tests read the reference's golden regression file with it.

    read_all(path) -> {"group/sub/dataset": numpy array, ...}
"""

import struct

import numpy as np

SIGNATURE = b"\x89HDF\r\n\x1a\n"
UNDEF = 0xFFFFFFFFFFFFFFFF


class H5File:
    def __init__(self, path):
        with open(path, "rb") as f:
            self.b = f.read()
        base = self.b.find(SIGNATURE)
        if base < 0:
            raise ValueError("not an HDF5 file")
        self.base = base
        s = base + 8
        version = self.b[s]
        if version != 0:
            raise ValueError(f"superblock version {version} not supported")
        self.so = self.b[s + 5]  # size of offsets
        self.sl = self.b[s + 6]  # size of lengths
        p = s + 8
        self.leaf_k, self.internal_k = struct.unpack_from("<HH", self.b, p)
        p += 4 + 4  # group leaf/internal K, file consistency flags
        self.base_address = self._off(p)
        p += 4 * self.so  # base, free-space, end-of-file, driver addresses
        # root group symbol table entry
        self.root = self._symbol_entry(p)

    # ---- primitive readers -------------------------------------------------
    def _uint(self, p, n):
        return int.from_bytes(self.b[p:p + n], "little")

    def _off(self, p):
        return self._uint(p, self.so)

    def _len(self, p):
        return self._uint(p, self.sl)

    def _addr(self, a):
        return self.base_address + a

    def _symbol_entry(self, p):
        name_off = self._off(p)
        header = self._off(p + self.so)
        cache = self._uint(p + 2 * self.so, 4)
        scratch = p + 2 * self.so + 8
        btree = heap = None
        if cache == 1:
            btree = self._off(scratch)
            heap = self._off(scratch + self.so)
        return {"name_off": name_off, "header": header, "cache": cache,
                "btree": btree, "heap": heap}

    def _entry_size(self):
        return 2 * self.so + 8 + 16

    # ---- local heap, B-tree, symbol nodes -----------------------------------
    def _heap_data(self, heap_addr):
        p = self._addr(heap_addr)
        if self.b[p:p + 4] != b"HEAP":
            raise ValueError("bad local heap")
        q = p + 8 + 2 * self.sl  # signature, version, reserved, data size, free list
        return self._addr(self._off(q))

    def _heap_name(self, data_addr, off):
        p = data_addr + off
        end = self.b.index(b"\0", p)
        return self.b[p:end].decode()

    def _group_entries(self, btree_addr, heap_addr):
        """(name, symbol entry) of every link of a symbol-table group."""
        data = self._heap_data(heap_addr)
        out = []
        stack = [btree_addr]
        while stack:
            p = self._addr(stack.pop())
            if self.b[p:p + 4] != b"TREE":
                raise ValueError("bad B-tree node")
            node_type, level = self.b[p + 4], self.b[p + 5]
            used = self._uint(p + 6, 2)
            if node_type != 0:
                raise ValueError("not a group B-tree")
            q = p + 8 + 2 * self.so  # skip left / right sibling addresses
            children = []
            for i in range(used):
                q += self.sl          # key i (heap offset)
                children.append(self._off(q))
                q += self.so
            if level > 0:
                stack.extend(reversed(children))
                continue
            for child in children:
                s = self._addr(child)
                if self.b[s:s + 4] != b"SNOD":
                    raise ValueError("bad symbol table node")
                n = self._uint(s + 6, 2)
                e = s + 8
                for _ in range(n):
                    ent = self._symbol_entry(e)
                    out.append((self._heap_name(data, ent["name_off"]), ent))
                    e += self._entry_size()
        return out

    # ---- object headers ------------------------------------------------------
    def _messages(self, header_addr):
        """(type, body offset, size) of every message of a v1 object header,
        continuation blocks included."""
        p = self._addr(header_addr)
        if self.b[p] != 1:
            raise ValueError(f"object header version {self.b[p]} not supported")
        n_msgs = self._uint(p + 2, 2)
        size = self._uint(p + 8, 4)
        blocks = [(p + 16, size)]  # header prefix is 12 bytes, padded to 16
        msgs = []
        while blocks and len(msgs) < n_msgs:
            q, size = blocks.pop(0)
            end = q + size
            while q + 8 <= end and len(msgs) < n_msgs:
                mtype = self._uint(q, 2)
                msize = self._uint(q + 2, 2)
                body = q + 8
                if mtype == 0x0010:  # continuation: offset, length
                    blocks.append((self._addr(self._off(body)), self._len(body + self.so)))
                msgs.append((mtype, body, msize))
                q = body + msize
        return msgs

    # ---- datasets ------------------------------------------------------------
    def _dataspace(self, p):
        version, ndim, flags = self.b[p], self.b[p + 1], self.b[p + 2]
        q = p + (8 if version == 1 else 4)
        return tuple(self._len(q + i * self.sl) for i in range(ndim))

    def _datatype(self, p):
        cls = self.b[p] & 0x0F
        bits = self.b[p + 1] | (self.b[p + 2] << 8) | (self.b[p + 3] << 16)
        size = self._uint(p + 4, 4)
        order = ">" if bits & 1 else "<"
        if cls == 0:  # fixed-point
            kind = "i" if bits & 0x08 else "u"
        elif cls == 1:  # IEEE floating point
            kind = "f"
        else:
            raise ValueError(f"datatype class {cls} not supported")
        return np.dtype(f"{order}{kind}{size}")

    def _layout(self, p):
        version = self.b[p]
        if version == 3:
            cls = self.b[p + 1]
            if cls == 0:  # compact: size, raw data
                n = self._uint(p + 2, 2)
                return ("compact", p + 4, n)
            if cls == 1:  # contiguous: address, size
                return ("contiguous", self._off(p + 2), self._len(p + 2 + self.so))
            raise ValueError("chunked datasets not supported")
        if version in (1, 2):
            ndim, cls = self.b[p + 1], self.b[p + 2]
            q = p + 8
            if cls == 1:
                return ("contiguous", self._off(q), None)
            if cls == 0:
                q += 4 * ndim  # dimension sizes
                n = self._uint(q, 4)
                return ("compact", q + 4, n)
            raise ValueError("chunked datasets not supported")
        raise ValueError(f"layout version {version} not supported")

    def _dataset(self, header_addr):
        shape = dtype = layout = None
        for mtype, body, _ in self._messages(header_addr):
            if mtype == 0x0001:
                shape = self._dataspace(body)
            elif mtype == 0x0003:
                dtype = self._datatype(body)
            elif mtype == 0x0008:
                layout = self._layout(body)
        if shape is None or dtype is None or layout is None:
            return None
        n = int(np.prod(shape)) if shape else 1
        nbytes = n * dtype.itemsize
        kind, at, _ = layout
        if kind == "contiguous":
            if at == UNDEF:  # never written: fill value, taken as zeros
                return np.zeros(shape, dtype)
            at = self._addr(at)
        raw = self.b[at:at + nbytes]
        return np.frombuffer(raw, dtype=dtype).reshape(shape).astype(dtype.newbyteorder("="))

    def _group_of(self, header_addr):
        for mtype, body, _ in self._messages(header_addr):
            if mtype == 0x0011:  # symbol table: B-tree, local heap
                return self._off(body), self._off(body + self.so)
        return None

    def read_all(self):
        out = {}
        root = self.root
        stack = [("", root["header"])]
        while stack:
            path, header = stack.pop()
            grp = self._group_of(header)
            if grp is None:
                ds = self._dataset(header)
                if ds is not None:
                    out[path] = ds
                continue
            for name, ent in self._group_entries(*grp):
                stack.append((f"{path}/{name}" if path else name, ent["header"]))
        return out


def read_all(path):
    return H5File(path).read_all()
