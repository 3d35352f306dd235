"""Headless VTK XML output of the SWE cell state.

The cell-data output of the reference's XML writer (src/SWE/SWE_xml_output.f90:94-121,
order-0 elements): one piece (.vtu) per call with one triangle per cell, three
points per cell (points are not shared between cells, as in the reference), cell
data "water height", "bathymetry", "momentum" (3 components, the third 0),
"rank", "section index", "depth" and "refinement flag", a field "time", and a
parallel index (.pvtu) that lists the pieces. The data is written as ASCII, as
the reference writes it. Nothing here touches the GPU: the state is whatever
the caller downloaded.
"""
import os

import numpy as np

from . import _lib
from .swe import _p


def uniform_vertices(depth):
    """Vertices of the cells of the uniform mesh at reference depth ``depth``, in
    traversal order, in the unit square: float64[n, 3, 2]."""
    n = 2 << depth
    v = np.empty((n, 3, 2), np.float64)
    _lib.check(_lib.load().swe_mesh_uniform_vertices(depth, _p(v)))
    return v


def world(vertices, cfg):
    """Unit-square coordinates to world coordinates: x * scaling + offset."""
    return vertices * cfg.scaling + np.asarray(cfg.offset, np.float64)


def _ascii(a, fmt):
    return "\n".join(" ".join(fmt % x for x in row) for row in np.asarray(a).reshape(len(a), -1))


def write_vtu(path, vertices, h, hu, hv, b, depth, flags=None, time=0.0, rank=0, section=1):
    """One unstructured-grid piece: vertices float64[n, 3, 2] (world coordinates),
    the state arrays float64[n], depth int8[n], flags int8[n] (zeros if None)."""
    n = len(h)
    if vertices.shape != (n, 3, 2):
        raise ValueError("vertices must have shape (n_cells, 3, 2)")
    flags = np.zeros(n, np.int8) if flags is None else np.asarray(flags)
    pts = np.concatenate([vertices.reshape(3 * n, 2), np.zeros((3 * n, 1))], axis=1)
    conn = np.arange(3 * n, dtype=np.int64).reshape(n, 3)
    offs = 3 * np.arange(1, n + 1, dtype=np.int64)
    mom = np.stack([hu, hv, np.zeros(n)], axis=1)
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="UnstructuredGrid" version="0.1" byte_order="LittleEndian">\n')
        f.write('<UnstructuredGrid>\n<FieldData>\n')
        f.write('<DataArray type="Float64" Name="time" NumberOfTuples="1" format="ascii">%.17g</DataArray>\n' % time)
        f.write('</FieldData>\n<Piece NumberOfPoints="%d" NumberOfCells="%d">\n' % (3 * n, n))
        f.write('<CellData>\n')
        for name, arr, typ, fmt, nc in (("water height", h, "Float64", "%.17g", 1),
                                        ("bathymetry", b, "Float64", "%.17g", 1),
                                        ("momentum", mom, "Float64", "%.17g", 3),
                                        ("rank", np.full(n, rank), "Int32", "%d", 1),
                                        ("section index", np.full(n, section), "Int32", "%d", 1),
                                        ("depth", depth, "Int8", "%d", 1),
                                        ("refinement flag", flags, "Int8", "%d", 1)):
            f.write('<DataArray type="%s" Name="%s" NumberOfComponents="%d" format="ascii">\n' % (typ, name, nc))
            f.write(_ascii(np.asarray(arr).reshape(n, nc), fmt))
            f.write('\n</DataArray>\n')
        f.write('</CellData>\n<Points>\n<DataArray type="Float64" NumberOfComponents="3" format="ascii">\n')
        f.write(_ascii(pts, "%.17g"))
        f.write('\n</DataArray>\n</Points>\n<Cells>\n')
        f.write('<DataArray type="Int64" Name="connectivity" format="ascii">\n' + _ascii(conn, "%d") + '\n</DataArray>\n')
        f.write('<DataArray type="Int64" Name="offsets" format="ascii">\n' + _ascii(offs.reshape(n, 1), "%d") +
                '\n</DataArray>\n')
        f.write('<DataArray type="UInt8" Name="types" format="ascii">\n' + _ascii(np.full((n, 1), 5), "%d") +
                '\n</DataArray>\n')
        f.write('</Cells>\n</Piece>\n</UnstructuredGrid>\n</VTKFile>\n')


def write_pvtu(path, pieces):
    """The parallel index of the reference's post_traversal_grid_op: the cell-data
    layout and the piece files (names relative to the index)."""
    with open(path, "w") as f:
        f.write('<?xml version="1.0"?>\n<VTKFile type="PUnstructuredGrid" version="0.1" byte_order="LittleEndian">\n')
        f.write('<PUnstructuredGrid GhostLevel="0">\n<PCellData>\n')
        for name, typ, nc in (("water height", "Float64", 1), ("bathymetry", "Float64", 1),
                              ("momentum", "Float64", 3), ("rank", "Int32", 1), ("section index", "Int32", 1),
                              ("depth", "Int8", 1), ("refinement flag", "Int8", 1)):
            f.write('<PDataArray type="%s" Name="%s" NumberOfComponents="%d"/>\n' % (typ, name, nc))
        f.write('</PCellData>\n<PPoints>\n<PDataArray type="Float64" NumberOfComponents="3"/>\n</PPoints>\n')
        for p in pieces:
            f.write('<Piece Source="%s"/>\n' % os.path.basename(p))
        f.write('</PUnstructuredGrid>\n</VTKFile>\n')


def write_output(stamp, iteration, grid, cfg, vertices, flags=None):
    """The reference's file naming: <stamp>_<iteration>_r0_s1.vtu and <stamp>_<iteration>.pvtu."""
    piece = "%s_%d_r0_s1.vtu" % (stamp, iteration)
    write_vtu(piece, world(vertices, cfg), grid.h, grid.hu, grid.hv, grid.b, grid.mesh.depth, flags,
              grid.r_time)
    index = "%s_%d.pvtu" % (stamp, iteration)
    write_pvtu(index, [piece])
    return index
