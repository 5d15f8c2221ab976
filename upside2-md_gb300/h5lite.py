"""Python access to HDF5 `.up` files without h5py/PyTables.

Reading goes through the package's C++ reader (``csrc/h5lite.cpp``, loaded
from ``libupside_h5lite.so``); ``copy_file`` rewrites a file through the C++
writer (``csrc/h5lite_write.cpp``) that the upside driver logs with.
``H5Writer`` below is a pure-Python writer for configurations: the
writer emits the same conservative subset the reader understands (superblock
v0, symbol-table groups, version-1 object headers, contiguous datasets,
version-1 attribute messages), which is also what HDF5 1.8+ libraries read.
"""
import ctypes
import os
import struct

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None


def _load():
    global _lib
    if _lib is None:
        path = os.path.join(_HERE, "libupside_h5lite.so")
        if not os.path.exists(path):
            raise RuntimeError("libupside_h5lite.so is not built; run __graft_entry__.build()")
        lib = ctypes.CDLL(path)
        lib.h5l_open.restype = ctypes.c_void_p
        lib.h5l_open.argtypes = [ctypes.c_char_p]
        lib.h5l_close.argtypes = [ctypes.c_void_p]
        lib.h5l_last_error.restype = ctypes.c_char_p
        lib.h5l_kind.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        lib.h5l_list.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_int]
        lib.h5l_attr_names.argtypes = lib.h5l_list.argtypes
        lib.h5l_shape.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64),
                                  ctypes.c_int, ctypes.POINTER(ctypes.c_int)]
        lib.h5l_attr_shape.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                       ctypes.POINTER(ctypes.c_int64), ctypes.c_int,
                                       ctypes.POINTER(ctypes.c_int)]
        lib.h5l_read_raw.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_void_p, ctypes.c_int64]
        lib.h5l_attr_read_raw.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_char_p,
                                          ctypes.c_void_p, ctypes.c_int64]
        lib.h5l_copy_file.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        _lib = lib
    return _lib


def copy_file(src, dst, skip=()):
    """Rewrite `src` as `dst` with the C++ writer, leaving out the paths in
    `skip` (datasets come out contiguous and uncompressed)."""
    if _load().h5l_copy_file(src.encode(), dst.encode(), "\n".join(skip).encode()):
        raise RuntimeError(_load().h5l_last_error().decode())


def _np_dtype(info):
    cls, size, signed, big = info
    order = ">" if big else "<"
    if cls == 0:
        return np.dtype("%s%s%d" % (order, "i" if signed else "u", size))
    if cls == 1:
        return np.dtype("%sf%d" % (order, size))
    if cls == 3:
        return np.dtype("S%d" % size)
    return np.dtype("V%d" % size)  # opaque bytes for classes the engine never reads


class H5File:
    """Read-only handle on an HDF5 file."""

    def __init__(self, path):
        lib = _load()
        self._lib = lib
        self._h = lib.h5l_open(os.fsencode(path))
        if not self._h:
            raise IOError(lib.h5l_last_error().decode())

    def close(self):
        if self._h:
            self._lib.h5l_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _err(self):
        raise KeyError(self._lib.h5l_last_error().decode())

    def kind(self, path):
        return self._lib.h5l_kind(self._h, path.encode())

    def exists(self, path):
        return self.kind(path) >= 0

    def _names(self, fn, *args):
        n = 1 << 16
        while True:
            buf = ctypes.create_string_buffer(n)
            r = fn(self._h, *args, buf, n)
            if r < 0:
                self._err()
            if r == 0:
                return [s for s in buf.value.decode().split("\n") if s]
            n = r

    def list(self, path):
        return self._names(self._lib.h5l_list, path.encode())

    def attr_names(self, path):
        return self._names(self._lib.h5l_attr_names, path.encode())

    def read(self, path):
        dims = (ctypes.c_int64 * 16)()
        info = (ctypes.c_int * 4)()
        rank = self._lib.h5l_shape(self._h, path.encode(), dims, 16, info)
        if rank < 0:
            self._err()
        dt = _np_dtype(tuple(info))
        shape = tuple(dims[i] for i in range(rank))
        out = np.empty(shape, dtype=dt)
        if self._lib.h5l_read_raw(self._h, path.encode(), out.ctypes.data, out.nbytes) < 0:
            self._err()
        return out

    def attr(self, path, name):
        dims = (ctypes.c_int64 * 16)()
        info = (ctypes.c_int * 5)()
        rank = self._lib.h5l_attr_shape(self._h, path.encode(), name.encode(), dims, 16, info)
        if rank < 0:
            self._err()
        if info[4] == 0:
            return None  # null dataspace
        dt = _np_dtype(tuple(info)[:4])
        shape = tuple(dims[i] for i in range(rank))
        out = np.empty(shape, dtype=dt)
        if self._lib.h5l_attr_read_raw(self._h, path.encode(), name.encode(), out.ctypes.data, out.nbytes) < 0:
            self._err()
        return out[()] if rank == 0 else out

    def attrs(self, path):
        return {n: self.attr(path, n) for n in self.attr_names(path)}


# --------------------------------------------------------------------------
# Writer
# --------------------------------------------------------------------------

_UNDEF = 0xFFFFFFFFFFFFFFFF


def _dtype_msg(dt):
    dt = np.dtype(dt)
    if dt.kind in "iu":
        flags = 0x08 if dt.kind == "i" else 0
        return struct.pack("<BBBBIHH", 0x10, flags, 0, 0, dt.itemsize, 0, dt.itemsize * 8)
    if dt.kind == "f":
        if dt.itemsize == 4:
            props = struct.pack("<HHBBBBI", 0, 32, 23, 8, 0, 23, 127)
            flags0 = 0x20
        else:
            props = struct.pack("<HHBBBBI", 0, 64, 52, 11, 0, 52, 1023)
            flags0 = 0x20
        return struct.pack("<BBBBI", 0x11, flags0, 0x1f if dt.itemsize == 4 else 0x3f, 0, dt.itemsize) + props
    if dt.kind == "S":
        return struct.pack("<BBBBI", 0x13, 0, 0, 0, dt.itemsize)
    raise ValueError("cannot write dtype %s" % dt)


def _dspace_msg(shape):
    rank = len(shape)
    return struct.pack("<BBBB4x", 1, rank, 0, 0) + b"".join(struct.pack("<Q", d) for d in shape)


def _pad8(b):
    return b + b"\0" * ((-len(b)) % 8)


def _normalize(value):
    if isinstance(value, (bytes, str)):
        v = value.encode() if isinstance(value, str) else value
        return np.array(v, dtype="S%d" % max(1, len(v)))
    arr = np.asarray(value)
    if arr.dtype.kind == "U":
        arr = arr.astype("S")
    if arr.dtype.kind == "b":
        arr = arr.astype(np.int8)
    if arr.dtype.kind == "f" and arr.dtype.itemsize not in (4, 8):
        arr = arr.astype(np.float64)
    if arr.dtype.byteorder == ">":
        arr = arr.astype(arr.dtype.newbyteorder("<"))
    return arr.copy(order="C")  # keeps 0-d scalars 0-d (ascontiguousarray would not)


class _Node:
    def __init__(self, is_group):
        self.is_group = is_group
        self.children = {}
        self.attrs = {}
        self.data = None


class H5Writer:
    """Build a tree of groups/datasets/attributes in memory, then ``save``.

    Paths use '/' separators; intermediate groups are created on demand.
    """

    def __init__(self):
        self.root = _Node(True)

    def _node(self, path, create_group=True):
        cur = self.root
        for part in [p for p in path.split("/") if p]:
            if part not in cur.children:
                if not create_group:
                    raise KeyError(path)
                cur.children[part] = _Node(True)
            cur = cur.children[part]
        return cur

    def group(self, path):
        return self._node(path)

    def dataset(self, path, value):
        parent, _, name = path.rstrip("/").rpartition("/")
        g = self._node(parent)
        n = _Node(False)
        n.data = _normalize(value)
        g.children[name] = n
        return n

    def set_attr(self, path, name, value):
        self._node(path, create_group=False).attrs[name] = _normalize(value)

    # -- serialisation -----------------------------------------------------
    def save(self, filename):
        out = bytearray()
        # superblock (96 bytes) + root symbol table entry, patched at the end
        out += b"\0" * 96

        def alloc(blob, align=8):
            while len(out) % align:
                out.append(0)
            addr = len(out)
            out.extend(blob)
            return addr

        def write_object(node):
            msgs = []
            if node.is_group:
                names = sorted(node.children)
                child_addrs = {nm: write_object(node.children[nm]) for nm in names}
                heap = bytearray(b"\0" * 8)  # offset 0: empty string (+padding)
                offs = {}
                for nm in names:
                    offs[nm] = len(heap)
                    heap += _pad8(nm.encode() + b"\0")
                heap_data_addr = alloc(bytes(heap))
                heap_hdr = b"HEAP" + bytes([0, 0, 0, 0]) + struct.pack("<QQQ", len(heap), _UNDEF, heap_data_addr)
                heap_addr = alloc(heap_hdr)
                # one symbol node holding every entry (group leaf K set large in the superblock)
                snod = bytearray(b"SNOD" + bytes([1, 0]) + struct.pack("<H", len(names)))
                for nm in names:
                    snod += struct.pack("<QQII16x", offs[nm], child_addrs[nm], 0, 0)
                snod += b"\0" * (40 * (2 * _LEAF_K - len(names)))
                snod_addr = alloc(bytes(snod))
                last_key = offs[names[-1]] if names else 0
                tree = b"TREE" + bytes([0, 0]) + struct.pack("<HQQ", 1 if names else 0, _UNDEF, _UNDEF)
                tree += struct.pack("<QQQ", 0, snod_addr, last_key)
                tree += b"\0" * ((2 * _INTERNAL_K) * 16)  # room for a full node
                tree_addr = alloc(tree)
                msgs.append((0x11, struct.pack("<QQ", tree_addr, heap_addr)))
            else:
                arr = node.data
                shape = arr.shape
                raw = arr.tobytes()
                data_addr = alloc(raw) if raw else _UNDEF
                msgs.append((0x01, _dspace_msg(shape)))
                msgs.append((0x03, _dtype_msg(arr.dtype)))
                layout = struct.pack("<BBQQ", 3, 1, data_addr, len(raw))
                msgs.append((0x08, layout))
            for name, val in node.attrs.items():
                nm = name.encode() + b"\0"
                dt = _dtype_msg(val.dtype)
                ds = _dspace_msg(val.shape)
                body = struct.pack("<BBHHH", 1, 0, len(nm), len(dt), len(ds))
                body += _pad8(nm) + _pad8(dt) + _pad8(ds) + val.tobytes()
                msgs.append((0x0C, body))
            blob = bytearray()
            for typ, body in msgs:
                body = _pad8(bytes(body))
                blob += struct.pack("<HHB3x", typ, len(body), 0) + body
            if not msgs:
                blob += struct.pack("<HHB3x", 0, 8, 0) + b"\0" * 8  # NIL message
            hdr = struct.pack("<BBHII4x", 1, 0, max(1, len(msgs)), 1, len(blob))
            return alloc(hdr + bytes(blob))

        root_addr = write_object(self.root)
        # root group's scratch pad caches its B-tree and heap addresses
        root_hdr = bytes(out[root_addr:root_addr + 64])
        msg_type = struct.unpack_from("<H", root_hdr, 16)[0]
        assert msg_type == 0x11
        tree_addr, heap_addr = struct.unpack_from("<QQ", root_hdr, 24)
        eof = len(out)
        sb = bytearray(b"\x89HDF\r\n\x1a\n")
        sb += bytes([0, 0, 0, 0, 0, 8, 8, 0])
        sb += struct.pack("<HHI", _LEAF_K, _INTERNAL_K, 0)
        sb += struct.pack("<QQQQ", 0, _UNDEF, eof, _UNDEF)
        sb += struct.pack("<QQII", 0, root_addr, 1, 0) + struct.pack("<QQ", tree_addr, heap_addr)
        out[0:len(sb)] = sb
        with open(filename, "wb") as f:
            f.write(bytes(out))


_LEAF_K = 512
_INTERNAL_K = 16
