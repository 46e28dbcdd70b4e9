"""The h5py-like reader of the driver's snapshots (fv3d_gb300.snapshots),
on a small run laid out as the driver writes it: raw float64 files and an
XDMF index with the vertex grid and, per save, rho / velocity (u, v, w
joined) / prs items at byte offsets."""
import numpy as np

from fv3d_gb300 import snapshots


def _item(name, seek, dims):
    return ('<DataItem Dimensions="%s" NumberType="Float" Precision="8" Format="Binary" Endian="Little" '
            'Seek="%d">%s</DataItem>' % (" ".join(str(d) for d in dims), seek, name))


def _fake_run(tmp_path, nx=6, ny=4, nz=1, times=(0.0, 0.25, 0.5)):
    nv = (nx + 1) * (ny + 1) * (nz + 1)
    nc = nx * ny * nz
    k, j, i = np.meshgrid(np.arange(nz + 1), np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
    grid = np.concatenate([(i * 0.1).ravel(), (j * 0.2).ravel(), (k * 1.0).ravel()])
    grid.tofile(str(tmp_path / "run_grid.bin"))
    rng = np.random.default_rng(5)
    states = []
    xml = ['<?xml version="1.0" ?>', '<Xdmf Version="2.0">', '<Domain CollectionType="Temporal">',
           '<Grid Name="MainTimeSeries" GridType="Collection" CollectionType="Temporal">',
           '<Topology Name="Main Topology" TopologyType="3DSMesh" NumberOfElements="%d %d %d"/>' % (nz + 1, ny + 1, nx + 1),
           '<Geometry Name="Main Geometry" GeometryType="X_Y_Z">']
    xml += [_item("run_grid.bin", a * nv * 8, (nz + 1, ny + 1, nx + 1)) for a in range(3)]
    xml.append("</Geometry>")
    for n, t in enumerate(times):
        q = rng.random((5, nz, ny, nx))
        states.append(q)
        name = "run_%04d.bin" % n
        q.tofile(str(tmp_path / name))
        xml.append('<Grid Name="Cells" GridType="Uniform"><Time TimeType="Single" Value="%.17g" />' % t)
        xml.append('<Attribute Name="rho" AttributeType="Scalar" Center="Cell">%s</Attribute>'
                   % _item(name, 0, (nz, ny, nx)))
        xml.append('<Attribute Name="velocity" AttributeType="Vector" Center="Cell">'
                   '<DataItem Dimensions="%d %d %d 3" ItemType="Function" Function="JOIN($0, $1, $2)">' % (nz, ny, nx)
                   + "".join(_item(name, v * nc * 8, (nz, ny, nx)) for v in (1, 2, 3)) + "</DataItem></Attribute>")
        xml.append('<Attribute Name="prs" AttributeType="Scalar" Center="Cell">%s</Attribute></Grid>'
                   % _item(name, 4 * nc * 8, (nz, ny, nx)))
    xml += ["</Grid>", "</Domain>", "</Xdmf>"]
    (tmp_path / "run.xdmf").write_text("\n".join(xml))
    return grid.reshape(3, nv), states


def test_reader_presents_the_reference_layout(tmp_path):
    grid, states = _fake_run(tmp_path)
    with snapshots.File(str(tmp_path / "run")) as f:
        assert f.keys() == ["x", "y", "z", "ite_0", "ite_1", "ite_2"]
        assert (f.attrs["Nx"], f.attrs["Ny"], f.attrs["Nz"], f.attrs["Ntx"]) == (6, 4, 1, 10)
        np.testing.assert_array_equal(f["x"], grid[0])
        np.testing.assert_array_equal(f["y"], grid[1])
        assert f["x"][1] - f["x"][0] == 0.1  # the tools' dx
        for n, q in enumerate(states):
            g = f["ite_%d" % n]
            assert g.attrs["time"] == (0.0, 0.25, 0.5)[n]
            for v, name in enumerate(("rho", "u", "v", "w", "prs")):
                np.testing.assert_array_equal(f["ite_%d/%s" % (n, name)], q[v])
                np.testing.assert_array_equal(g[name], q[v])
    assert snapshots.File(str(tmp_path / "run.xdmf")).keys()[-1] == "ite_2"
