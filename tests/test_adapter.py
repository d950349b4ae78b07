"""The DROPS drop-in shim (drops_gb300/adapter/tracefem_drops.{h,cpp}) compiled against the reference's own
headers and linked with its objects (oracle/build_ref.sh builds oracle/_ref/adapter_check where the DROPS
sources exist; skipped elsewhere).  On a machine without a GPU the shim must refuse loudly: there is no CPU
fallback."""
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
from oracle import pyoracle as O  # noqa: E402
from tfg import read_tfg  # noqa: E402

CHECK = os.path.join(ROOT, "oracle", "_ref", "adapter_check")
pytestmark = pytest.mark.skipif(not os.path.exists(CHECK), reason="adapter_check not built (no DROPS sources)")


def test_flatten_matches_this_librarys_mesh(tmp_path):
    """Flatten(mg, level): vertices in triangulation order with the reference's coordinates, tets with the
    geom/topo.cpp vertex and edge order; the level-set values per vertex and per edge."""
    n, a = 8, 5.0 / 3.0
    out = tmp_path / "flat.bin"
    subprocess.run([CHECK, "flatten", str(n), repr(a), str(out)], check=True, capture_output=True)
    d = read_tfg(str(out))
    mesh = O.brick(n, a=a)
    assert np.array_equal(d["coords"], mesh.coords.ravel())
    assert np.array_equal(d["tet_v"], mesh.tet_v.astype(np.int64).ravel())
    # edges: the shim numbers them in the triangulation's edge order; match them by their vertex pairs
    ev = d["edge_v"].reshape(-1, 2)
    tet_pairs = np.sort(ev[d["tet_e"].reshape(-1, 6)], axis=2)
    assert np.array_equal(tet_pairs, np.sort(mesh.edge_v[mesh.tet_e], axis=2).astype(np.int64))
    lv, le = O.levelset(mesh, O.LS_SPHERE, [0, 0, 0, 1.0], p2=True)
    assert np.array_equal(d["ls_vert"], lv)
    key = {tuple(sorted(p)): i for i, p in enumerate(mesh.edge_v.tolist())}
    emap = np.array([key[tuple(sorted(p))] for p in ev.tolist()])
    assert np.array_equal(d["ls_edge"], le[emap])


def test_shim_fails_loudly_without_gpu():
    """gpu::DistributeDOFs on a machine with no usable GPU throws DROPSErrCL; with a GPU the same driver
    compares the shim's numbering, M/A/C_n and PCG solution with the reference's own calls."""
    r = subprocess.run([CHECK, "gpu", "8", repr(5.0 / 3.0)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("no-gpu: libtracefem") or r.stdout.strip() == "gpu: ok", r.stdout
