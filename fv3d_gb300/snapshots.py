"""Read the snapshots of an ``fv3d`` driver run the way the reference's HDF5
output is read.

The reference writes ``<filename_out>.h5`` (IOManager.h:88-190): root
attributes Nx, Ny, Nz, Ntx, ..., datasets ``x``, ``y``, ``z`` (vertex
coordinates, flattened in k, j, i order) and one group ``ite_<n>`` per save
holding ``rho``, ``u``, ``v``, ``w``, ``prs`` ([Nz][Ny][Nx]) with a ``time``
attribute; its Python tools (python/*.py) open it with ``h5py.File``.  The
``fv3d`` driver writes that file (``fv_h5_save``, ``--format h5``, the
default) or the same quantities as raw float64 files indexed by an XDMF file
(``--format raw``).  :class:`File` opens either with the h5py access pattern
the tools use -- ``f['x']``, ``f['ite_3/rho']``, ``f['ite_3'].attrs['time']``,
``f.keys()``, ``f.attrs`` -- so a tool runs with ``h5py.File(name, 'r')``
replaced by ``snapshots.File(name)`` where h5py is not installed.

The HDF5 reader here covers the original file format that libhdf5 writes by
default and ``fv_h5_save`` writes (superblock 0 or 1, version-1 object
headers with continuation blocks, symbol-table groups, contiguous or compact
datasets of IEEE floats, integers and fixed-length strings, version-1
attributes); other files raise ``NotImplementedError``.
"""
import mmap
import os
import struct
import xml.etree.ElementTree as ET

import numpy as np

__all__ = ["File", "Group", "H5File"]

_UNDEF = 0xFFFFFFFFFFFFFFFF


class H5File:
    """Read-only HDF5 file in the original format (see the module text)."""

    def __init__(self, path):
        self._f = open(path, "rb")
        self._m = mmap.mmap(self._f.fileno(), 0, access=mmap.ACCESS_READ)
        at = 0
        while self._m[at:at + 8] != b"\x89HDF\r\n\x1a\n":
            at = 512 if at == 0 else 2 * at  # user block sizes: 0, 512, 1024, ...
            if at + 8 > len(self._m):
                raise ValueError("%s: not an HDF5 file" % path)
        ver = self._m[at + 8]
        if ver not in (0, 1):
            raise NotImplementedError("HDF5 superblock version %d" % ver)
        if self._m[at + 13] != 8 or self._m[at + 14] != 8:
            raise NotImplementedError("HDF5 offsets / lengths other than 8 bytes")
        p = at + 24 + (4 if ver == 1 else 0)
        self._base = struct.unpack_from("<Q", self._m, p)[0]
        self.root = self._u64(p + 32 + 8)  # root entry: name offset, object header
        self.root_attrs = self.attributes(self.root)

    def close(self):
        if self._m is not None:
            self._m.close()
            self._f.close()
            self._m = None

    def _u64(self, p):
        return struct.unpack_from("<Q", self._m, p)[0]

    def _addr(self, a):
        return self._base + a

    def messages(self, header):
        """(type, bytes) of every message of the object header at `header`."""
        p = self._addr(header)
        if self._m[p] != 1:
            raise NotImplementedError("object header version %d" % self._m[p])
        n, _, size = struct.unpack_from("<HII", self._m, p + 2)
        chunks = [(p + 16, size)]
        out = []
        while chunks and len(out) < n:
            q, size = chunks.pop(0)
            end = q + size
            while q + 8 <= end and len(out) < n:
                mtype, msize = struct.unpack_from("<HH", self._m, q)
                body = bytes(self._m[q + 8:q + 8 + msize])
                if mtype == 0x10:  # continuation: another chunk of messages
                    a, length = struct.unpack_from("<QQ", body)
                    chunks.append((self._addr(a), length))
                out.append((mtype, body))
                q += 8 + msize
        return out

    def members(self, header):
        """{name: object header address} of the group at `header`."""
        stab = [b for t, b in self.messages(header) if t == 0x11]
        if not stab:
            raise NotImplementedError("group without a symbol table")
        btree, heap = struct.unpack_from("<QQ", stab[0])
        h = self._addr(heap)
        if self._m[h:h + 4] != b"HEAP":
            raise ValueError("bad local heap")
        dsize, _, daddr = struct.unpack_from("<QQQ", self._m, h + 8)
        names = self._m[self._addr(daddr):self._addr(daddr) + dsize]
        out = {}
        self._walk(btree, names, out)
        return out

    def _walk(self, node, names, out):
        p = self._addr(node)
        if self._m[p:p + 4] != b"TREE" or self._m[p + 4] != 0:
            raise ValueError("bad group B-tree node")
        level = self._m[p + 5]
        used = struct.unpack_from("<H", self._m, p + 6)[0]
        for c in range(used):
            child = self._u64(p + 32 + 16 * c)
            if level > 0:
                self._walk(child, names, out)
                continue
            s = self._addr(child)
            if self._m[s:s + 4] != b"SNOD":
                raise ValueError("bad symbol-table node")
            for e in range(struct.unpack_from("<H", self._m, s + 6)[0]):
                off, hdr = struct.unpack_from("<QQ", self._m, s + 8 + 40 * e)
                end = names.find(b"\0", off)
                out[names[off:end].decode()] = hdr

    @staticmethod
    def _dtype(b):
        cls, ver = b[0] & 0x0F, b[0] >> 4
        flags = b[1] | (b[2] << 8) | (b[3] << 16)
        size = struct.unpack_from("<I", b, 4)[0]
        order = ">" if flags & 1 else "<"
        if cls == 0:
            return np.dtype("%s%s%d" % (order, "i" if flags & 8 else "u", size))
        if cls == 1 and size in (4, 8):
            return np.dtype("%sf%d" % (order, size))
        if cls == 3:
            return np.dtype("S%d" % size)
        raise NotImplementedError("HDF5 datatype class %d version %d" % (cls, ver))

    @staticmethod
    def _shape(b):
        ver, rank = b[0], b[1]
        q = 8 if ver == 1 else 4
        if ver == 2 and b[3] == 0:
            return ()
        return tuple(struct.unpack_from("<%dQ" % rank, b, q)) if rank else ()

    def attributes(self, header):
        out = {}
        for t, b in self.messages(header):
            if t != 0x0C:
                continue
            if b[0] != 1:
                raise NotImplementedError("attribute message version %d" % b[0])
            nlen, tlen, slen = struct.unpack_from("<HHH", b, 2)
            al = lambda n: (n + 7) & ~7  # noqa: E731
            q = 8
            name = b[q:q + nlen].split(b"\0")[0].decode()
            q += al(nlen)
            dt = self._dtype(b[q:q + tlen])
            q += al(tlen)
            shape = self._shape(b[q:q + slen])
            q += al(slen)
            count = int(np.prod(shape)) if shape else 1
            val = np.frombuffer(b, dtype=dt, count=count, offset=q).reshape(shape)
            out[name] = val[()] if shape == () else val.copy()
        return out

    def dataset(self, header):
        msgs = dict(self.messages(header))
        dt, shape = self._dtype(msgs[0x3]), self._shape(msgs[0x1])
        lay = msgs[0x8]
        count = int(np.prod(shape)) if shape else 1
        if lay[0] == 3 and lay[1] == 1:  # contiguous
            addr = struct.unpack_from("<Q", lay, 2)[0]
        elif lay[0] == 3 and lay[1] == 0:  # compact
            return np.frombuffer(lay, dtype=dt, count=count, offset=4).reshape(shape).copy()
        elif lay[0] in (1, 2) and lay[2] == 1:
            addr = struct.unpack_from("<Q", lay, 8)[0]
        else:
            raise NotImplementedError("HDF5 data layout version %d class %d" % (lay[0], lay[1]))
        if addr == _UNDEF:
            return np.zeros(shape, dt)
        return np.frombuffer(self._m, dtype=dt, count=count, offset=self._addr(addr)).reshape(shape).copy()

    def is_group(self, header):
        return any(t == 0x11 for t, _ in self.messages(header))


class _H5Group:
    """A group of an HDF5 file, h5py-like: keys(), [name], attrs."""

    def __init__(self, h5, header):
        self._h5 = h5
        self._members = h5.members(header)
        self.attrs = h5.attributes(header)

    def keys(self):
        return list(self._members)

    def __contains__(self, name):
        return name.strip("/").partition("/")[0] in self._members

    def __len__(self):
        return len(self._members)

    def __getitem__(self, key):
        head, _, rest = key.strip("/").partition("/")
        hdr = self._members[head]
        if self._h5.is_group(hdr):
            g = _H5Group(self._h5, hdr)
            return g[rest] if rest else g
        if rest:
            raise KeyError(key)
        return self._h5.dataset(hdr)


def _read_item(base, item):
    """The float64 array a Binary DataItem of the index points at."""
    dims = tuple(int(v) for v in item.get("Dimensions").split())
    count = int(np.prod(dims))
    path = os.path.join(base, item.text.strip())
    return np.fromfile(path, dtype=np.float64, count=count, offset=int(item.get("Seek", "0"))).reshape(dims)


class Group:
    """One save (``ite_<n>``): its fields and its ``time`` attribute."""

    def __init__(self, base, grid):
        self._base = base
        self.attrs = {"time": float(grid.find("Time").get("Value"))}
        self._items = {}
        for att in grid.findall("Attribute"):
            name = att.get("Name")
            if name == "velocity":
                parts = att.findall("DataItem/DataItem")
                for comp, item in zip(("u", "v", "w"), parts):
                    self._items[comp] = item
            else:
                self._items[name] = att.find("DataItem")

    def keys(self):
        return ["prs", "rho", "u", "v", "w"]

    def __contains__(self, name):
        return name in self._items

    def __getitem__(self, name):
        if name not in self._items:
            raise KeyError(name)
        return _read_item(self._base, self._items[name])


class File:
    """Read-only, h5py-like view of a run: an HDF5 file (a path ending in
    ``.h5``, or ``prefix`` with ``prefix.h5`` present) or the raw snapshots
    written under ``prefix`` (the driver's ``--out``; a path to the
    ``.xdmf`` file is accepted too)."""

    def __new__(cls, prefix, mode="r"):
        if mode != "r":
            raise ValueError("snapshots are read-only")
        h5 = prefix if prefix.endswith(".h5") else prefix + ".h5"
        if prefix.endswith(".h5") or (not prefix.endswith(".xdmf") and os.path.exists(h5)):
            return _H5Root(h5)
        return super().__new__(cls)

    def __init__(self, prefix, mode="r"):
        xdmf = prefix if prefix.endswith(".xdmf") else prefix + ".xdmf"
        self._base = os.path.dirname(os.path.abspath(xdmf))
        root = ET.parse(xdmf).getroot()
        coll = root.find("Domain/Grid")
        nz1, ny1, nx1 = (int(v) for v in coll.find("Topology").get("NumberOfElements").split())
        self._geo = coll.findall("Geometry/DataItem")
        self._groups = [Group(self._base, g) for g in coll.findall("Grid")]
        nx, ny, nz = nx1 - 1, ny1 - 1, nz1 - 1
        ng = 2
        self.attrs = {"Nx": nx, "Ny": ny, "Nz": nz, "Ntx": nx + 2 * ng, "Nty": ny + 2 * ng, "Ntz": nz + 2 * ng,
                      "ibeg": ng, "iend": ng + nx, "jbeg": ng, "jend": ng + ny, "kbeg": ng, "kend": ng + nz}

    def keys(self):
        return ["x", "y", "z"] + ["ite_%d" % i for i in range(len(self._groups))]

    def __len__(self):
        return len(self.keys())

    def __contains__(self, key):
        return key in self.keys()

    def __getitem__(self, key):
        key = key.strip("/")
        if key in ("x", "y", "z"):
            return _read_item(self._base, self._geo["xyz".index(key)]).ravel()
        head, _, rest = key.partition("/")
        if not head.startswith("ite_"):
            raise KeyError(key)
        g = self._groups[int(head[4:])]
        return g[rest] if rest else g

    def close(self):
        pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False


class _H5Root(_H5Group):
    """The root group of an HDF5 file, with close() and a context manager."""

    def __init__(self, path):
        self._file = H5File(path)
        super().__init__(self._file, self._file.root)

    def close(self):
        self._file.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
        return False
