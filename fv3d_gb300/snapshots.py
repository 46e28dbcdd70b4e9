"""Read the snapshots of an ``fv3d`` driver run the way the reference's HDF5
output is read.

The reference writes ``<filename_out>.h5`` (IOManager.h:88-190): root
attributes Nx, Ny, Nz, Ntx, ..., datasets ``x``, ``y``, ``z`` (vertex
coordinates, flattened in k, j, i order) and one group ``ite_<n>`` per save
holding ``rho``, ``u``, ``v``, ``w``, ``prs`` ([Nz][Ny][Nx]) with a ``time``
attribute; its Python tools (python/*.py) open it with ``h5py.File``.  The
``fv3d`` driver writes the same quantities as raw float64 files indexed by
an XDMF file (``<prefix>.xdmf``).  :class:`File` presents that run with the
h5py access pattern the tools use -- ``f['x']``, ``f['ite_3/rho']``,
``f['ite_3'].attrs['time']``, ``f.keys()``, ``f.attrs`` -- so a tool runs
with ``h5py.File(name, 'r')`` replaced by ``snapshots.File(prefix)``.
"""
import os
import xml.etree.ElementTree as ET

import numpy as np

__all__ = ["File", "Group"]


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
    """Read-only, h5py-like view of the run written under ``prefix`` (the
    driver's ``--out``; a path to the ``.xdmf`` file is accepted too)."""

    def __init__(self, prefix, mode="r"):
        if mode != "r":
            raise ValueError("snapshots are read-only")
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
