"""VTK output (GPU): the reference writer's layout, synchronous and from snapshots.

* The data blocks of wf_write_vtk match those the reference's own VTKWriter
  printed for the same state (tests/golden/vtk_*.npz, written by
  tests/golden/gen_golden.py from the reference compiled from its sources):
  the FP64 step equals the reference to 1e-9, the reference prints 5 or 6
  significant digits, so each block is held to 1e-3 of its largest value
  (+1e-4 absolute for the fixed-point ContForce block). Blocks the reference
  fills from uninitialised arrays without contact (ext_nodes, nod_area,
  ele_area) are compared only where they are computed.
* A series of snapshots (wf_snapshot, written with wf_write_snapshot_vtk while
  later steps run) gives the same files, byte for byte, as wf_write_vtk called
  at the same steps.
"""
import os

import numpy as np
import pytest

import weldformfem_gb300 as wf
from tests import helpers as H
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu

GOLDEN = H.GOLDEN


def vtk_cases():
    """The cases of tests/golden/gen_golden.py's VTK fixtures."""
    import importlib.util

    spec = importlib.util.spec_from_file_location("gen_golden",
                                                  os.path.join(GOLDEN, "gen_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.vtk_cases()


@pytest.mark.parametrize("name,case,steps,extra", vtk_cases(), ids=[c[0] for c in vtk_cases()])
def test_vtk_blocks_match_reference_writer(tmp_path, name, case, steps, extra):
    g = dict(np.load(os.path.join(GOLDEN, f"{name}.npz")))
    d = wf.Domain(wf.WF_FP64)
    H.setup(d, case, extra)
    d.init()
    d.run(steps)
    out = tmp_path / "gpu.vtk"
    d.write_vtk(str(out))
    ours = {f"{sec}/{nm}": v for (sec, nm), v in H.parse_vtk(str(out)).items()}
    skip = {"steps", "cell/ele_area"}
    if "die" not in extra:
        skip |= {"point/ext_nodes", "point/nod_area"}
    compared = 0
    for key, ref in g.items():
        if key in skip:
            continue
        assert key in ours, key
        got = ours[key]
        assert got.shape == ref.shape, (key, got.shape, ref.shape)
        if key == "cells/CELLS":
            np.testing.assert_array_equal(got, ref)
        else:
            err = float(np.max(np.abs(got - ref))) if ref.size else 0.0
            tol = 1e-3 * float(np.max(np.abs(ref))) + 1e-4
            assert err <= tol, (key, err, tol)
        compared += 1
    assert compared >= 20


def series(tmp_path, tag, prec, case, extra, snapshots):
    """Writes four outputs 40 steps apart, with snapshots or synchronously."""
    d = wf.Domain(prec)
    H.setup(d, case, extra)
    d.init()
    files, pending = [], None
    for i in range(4):
        d.run(40)
        path = str(tmp_path / f"{tag}_{i}.vtk")
        if snapshots:
            slot = d.snapshot()                 # queued behind the 40 steps
            if pending is not None:
                d.write_snapshot_vtk(*pending)  # the previous one, while this copies
            pending = (slot, path)
        else:
            d.write_vtk(path)
        files.append(path)
    if snapshots:
        d.write_snapshot_vtk(*pending)
    d.sync()
    return files


@pytest.mark.parametrize("prec", [wf.WF_FP64, wf.WF_MIXED], ids=["fp64", "mixed"])
def test_snapshot_series_equals_synchronous_writes(tmp_path, prec):
    name, case, steps, extra = vtk_cases()[1]        # tetrahedra under a moving die
    a = series(tmp_path, "snap", prec, case, extra, True)
    b = series(tmp_path, "sync", prec, case, extra, False)
    for fa, fb in zip(a, b):
        assert open(fa, "rb").read() == open(fb, "rb").read(), fa
    blocks = H.parse_vtk(a[-1])
    assert ("point", "DISP") in blocks and blocks[("point", "DISP")].any()


def test_snapshot_slots():
    case = W.config(0, scale=(6, 6, 6))
    d = wf.Domain(wf.WF_MIXED)
    W.apply(d, case)
    d.init()
    s0 = d.snapshot()
    d.run(10)
    s1 = d.snapshot()
    assert {s0, s1} == {0, 1}
    with pytest.raises(wf.WfError) as e:
        d.snapshot()                            # both slots hold unwritten states
    assert e.value.status == wf.WF_ERR_STATE
    with pytest.raises(wf.WfError):
        d.write_snapshot_vtk(5, "/dev/null")    # no such slot
