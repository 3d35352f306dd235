"""CPU tests of the C ABI library: it loads, exports every entry point that
include/samoa_swe.h declares, builds the reference mesh, and rejects corrupt
meshes with an error code (no compute on a GPU here)."""
import ctypes as C
import json
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from oracle import oracle as O
from samoa_gb300 import _lib, swe

from .conftest import HAS_GPU, ROOT


def _header_functions():
    with open(os.path.join(ROOT, "include", "samoa_swe.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^int\s+(swe_\w+)\s*\(", text, re.M)))


def test_exports_every_declared_symbol(swe_lib):
    names = _header_functions()
    assert len(names) >= 15
    for n in names:
        assert hasattr(swe_lib, n), n
    assert sorted(_lib.EXPORTS) == names


def test_params_layout_matches_oracle():
    assert C.sizeof(_lib.SweParams) == C.sizeof(O.Params)
    for (a, ta), (b, tb) in zip(_lib.SweParams._fields_, O.Params._fields_):
        assert a == b and ta == tb


@pytest.mark.parametrize("depth", range(0, 13))
def test_uniform_mesh_matches_oracle(swe_lib, oracle_lib, depth):
    """Bit-exact SFC order, plotter types and edge indexing against the oracle's
    restatement of init_grid and the traversal's stack walk."""
    m = swe.uniform_mesh(depth)
    o = O.mesh_uniform(depth)
    assert np.array_equal(m.depth, o["cells5"][:, 1])
    assert np.array_equal(m.plotter, o["cells5"][:, 2])
    assert np.array_equal(m.edge_cells, o["edge_cells"])
    assert np.array_equal(m.edge_local, o["edge_local"])
    assert np.array_equal(m.bnd_cell, o["bnd_cell"])
    assert np.array_equal(m.bnd_local, o["bnd_local"])
    assert np.abs(m.centroids - o["coords"].mean(1)).max() < 1e-15


def _validate(m, **over):
    d = over.get("depth", m.depth)
    p = over.get("plotter", m.plotter)
    ec = np.ascontiguousarray(over.get("edge_cells", m.edge_cells), np.int64)
    el = np.ascontiguousarray(over.get("edge_local", m.edge_local), np.int8)
    bc = np.ascontiguousarray(over.get("bnd_cell", m.bnd_cell), np.int64)
    bl = np.ascontiguousarray(over.get("bnd_local", m.bnd_local), np.int8)
    n = over.get("n", len(d))
    P = lambda a: a.ctypes.data_as(C.c_void_p)
    return _lib.load().swe_mesh_validate(n, P(np.ascontiguousarray(d)), P(np.ascontiguousarray(p)), len(ec), P(ec),
                                         P(el), len(bc), P(bc), P(bl))


@pytest.mark.parametrize("depth", [5, 20])
def test_mesh_validation_rejects_corrupt_streams(swe_lib, depth):
    """Corrupt streams are rejected with the first bad item named; at depth 20
    (2^21 cells) the check runs in parts on host threads."""
    m = swe.uniform_mesh(depth)
    assert _validate(m) == 0
    bad = m.edge_cells.copy()
    bad[3, 1] = m.n_cells + 5
    assert _validate(m, edge_cells=bad) == -1
    assert "invalid" in _lib.last_error()
    bad = m.edge_cells.copy()
    bad[4, 0] = bad[4, 1]
    assert _validate(m, edge_cells=bad) == -1
    bad = m.edge_local.copy()
    bad[2, 0] = 4
    assert _validate(m, edge_local=bad) == -1
    dup = m.edge_local.copy()
    dup[0] = dup[1]
    dupc = m.edge_cells.copy()
    dupc[0] = dupc[1]
    assert _validate(m, edge_local=dup, edge_cells=dupc) == -1
    assert "used twice" in _lib.last_error()
    k = len(m.edge_cells) - 2  # a duplicate claim at the far end of the list (another part)
    dup = m.edge_local.copy()
    dup[k] = dup[3]
    dupc = m.edge_cells.copy()
    dupc[k] = dupc[3]
    assert _validate(m, edge_local=dup, edge_cells=dupc) == -1
    assert _lib.last_error() == "edge %d: a cell's local edge is used twice" % k
    p = m.plotter.copy()
    p[7] = 0
    assert _validate(m, plotter=p) == -1
    d = m.depth.copy()
    d[1] = 61
    assert _validate(m, depth=d) == -1
    assert _validate(m, bnd_cell=m.bnd_cell[:-1], bnd_local=m.bnd_local[:-1]) == -1
    bc = m.bnd_cell.copy()
    bc[0] = -1
    assert _validate(m, bnd_cell=bc) == -1


def test_mesh_uniform_rejects_bad_depth(swe_lib):
    n = C.c_int64()
    assert swe_lib.swe_mesh_uniform(-1, C.byref(n), None, None, *([None] * 7)) == -1
    assert swe_lib.swe_mesh_uniform(30, C.byref(n), None, None, *([None] * 7)) == -1


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU error path")
def test_create_without_gpu_reports_error(swe_lib):
    p = C.c_void_p()
    rc = swe_lib.swe_create(C.byref(p), 0)
    assert rc in (-1, -2) and not p.value
    assert _lib.last_error()


def test_null_arguments_are_errors(swe_lib):
    assert swe_lib.swe_traverse(None, 1) == -1
    assert swe_lib.swe_set_params(None, None) == -1
    assert swe_lib.swe_destroy(None) == 0
    # tuning calls on a null context report an error instead of touching memory
    assert swe_lib.swe_set_segment_order(None, 1) == -1
    assert swe_lib.swe_set_cross_pass(None, 0) == -1
    assert swe_lib.swe_set_tiling(None, 512, 128) == -1
    buf = C.create_string_buffer(8)
    assert swe_lib.swe_last_error(buf, 8) == 0


def test_initial_dt_matches_formula():
    m = swe.uniform_mesh(6)
    n = m.n_cells
    rng = np.random.default_rng(0)
    b = -rng.uniform(1, 5, n)
    h = b + rng.uniform(0, 3, n)
    hu, hv = rng.normal(size=n), rng.normal(size=n)
    dt = swe.initial_dt(m, h, hu, hv, b, 0.45)
    d = int(m.depth[0])
    depth = h - b
    s = np.sqrt(9.80665 * depth) + np.sqrt((hu * hu + hv * hv) / (depth * depth))
    edges = (O.leg_size(d) + O.leg_size(d - 1)) + O.leg_size(d)
    assert dt == 0.45 * (O.cell_volume(d) / (edges * s.max()))


def test_bench_reference_arm_json(tmp_path):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "2",
                          "--warmup", "1", "--log2-cells", "12"], capture_output=True, text=True, timeout=300,
                         cwd=ROOT)
    assert out.returncode == 0, out.stderr
    line = [l for l in out.stdout.splitlines() if l.startswith("{")][-1]
    j = json.loads(line)
    assert j["impl"] == "reference" and j["value"] > 0 and j["unit"] == "cell-updates/s"
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["cpu_baseline"]["kind"] == "port"
    assert j["config"]["cells"] == 1 << 12  # the whole workload, not a sample


def test_bench_reference_arm_loads_no_product_library():
    """The CPU arm builds its workload on the oracle's own mesh: the GPU library
    is never loaded, and the mesh equals the product's uniform mesh."""
    code = ("import sys; sys.path.insert(0, %r); import bench, numpy as np; "
            "s = bench.basin_from_oracle(10, 'fwave'); "
            "maps = open('/proc/self/maps').read(); "
            "print('LOADED' if 'libsamoa_swe' in maps else 'CLEAN', s.grid.mesh.n_cells)") % ROOT
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert out.returncode == 0, out.stderr
    assert out.stdout.split() == ["CLEAN", "1024"]


def test_bench_reference_arm_two_ranks_gloo():
    """Replicas path under torchrun with world size 2: rank 0 prints, rank 1 exits 0."""
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    out = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                          "--master-addr", "127.0.0.1", "--master-port", "29517", os.path.join(ROOT, "bench.py"),
                          "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
                          "--log2-cells", "10"], capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
