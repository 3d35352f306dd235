"""Headless VTK output: cell vertices of the uniform mesh and the XML files."""
import xml.etree.ElementTree as ET

import numpy as np

from samoa_gb300 import scenarios, swe, vtk


def test_uniform_vertices_match_mesh(swe_lib):
    m = swe.uniform_mesh(7)
    v = vtk.uniform_vertices(7)
    assert v.shape == (m.n_cells, 3, 2)
    assert np.allclose(v.mean(axis=1), m.centroids, rtol=0, atol=1e-15)
    # every cell has area 1 / n_cells (the two root triangles halve the unit square)
    a = 0.5 * np.abs((v[:, 1, 0] - v[:, 0, 0]) * (v[:, 2, 1] - v[:, 0, 1]) -
                     (v[:, 2, 0] - v[:, 0, 0]) * (v[:, 1, 1] - v[:, 0, 1]))
    assert np.allclose(a, 1.0 / m.n_cells)
    # an inner edge's two cells share both end points
    for (c0, c1), (l0, l1) in zip(m.edge_cells[:200], m.edge_local[:200]):
        s0 = {tuple(p) for p in v[c0]}
        s1 = {tuple(p) for p in v[c1]}
        assert len(s0 & s1) == 2


def test_write_vtu_and_pvtu(swe_lib, tmp_path):
    scn = scenarios.radial_dam_break(log2_cells=8, boundary="slip")
    g = scn.grid
    v = vtk.uniform_vertices(7)
    idx = vtk.write_output(str(tmp_path / "swe"), 3, g, scn.cfg, v)
    root = ET.parse(idx).getroot()
    assert root.attrib["type"] == "PUnstructuredGrid"
    src = root.find(".//Piece").attrib["Source"]
    piece = ET.parse(tmp_path / src).getroot()
    p = piece.find(".//Piece")
    assert int(p.attrib["NumberOfCells"]) == g.mesh.n_cells
    arrays = {a.attrib["Name"]: a for a in piece.iter("DataArray") if "Name" in a.attrib}
    h = np.array(arrays["water height"].text.split(), float)
    assert np.array_equal(h, g.h)
    mom = np.array(arrays["momentum"].text.split(), float).reshape(-1, 3)
    assert np.array_equal(mom[:, 0], g.hu)
    pts = np.array(piece.find(".//Points/DataArray").text.split(), float).reshape(-1, 3)
    assert np.allclose(pts[:, :2].reshape(-1, 3, 2), v * scn.cfg.scaling + np.asarray(scn.cfg.offset))
