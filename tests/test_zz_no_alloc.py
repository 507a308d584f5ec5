"""The allocation-free entry point, wf_nodal_volumes_noalloc (GPU).

It serves callers that may not allocate device memory: everything it needs is
passed in by the caller except its element-volume scratch, which lives in a
static device array inside the library. This test calls it through the C ABI
with inputs and output in device buffers the test owns, twice in a row on
different meshes (tetrahedra, then hexahedra, so the second call reuses the
scratch the first one left behind), and compares each result with the nodal
volumes the regular domain path (wf_init, wf_get_node_scalar) computes for
the same mesh, within the FP64 tolerance of the parity tests (1e-9 relative);
a repeated call must give the same bits. The file is collected last so a run
that stops at the first failure has run every other test first.
"""
import numpy as np
import pytest

import weldformfem_gb300 as wf
from weldformfem_gb300 import workloads as W

pytestmark = pytest.mark.gpu
TOL = 1e-9


def domain_voln(case):
    d = wf.Domain(wf.WF_FP64)
    W.apply(d, case)
    d.init()
    return d, d.node_scalar("voln")


def noalloc_voln(torch, case, d, stream=None):
    elnod, nodel, _loc, off, cnt = d.conn()
    nn, ne, npe = d.nn, d.ne, d.npe
    dev = torch.device("cuda:0")
    xyz = torch.from_numpy(np.ascontiguousarray(case.coords().reshape(-1))).to(dev)
    el = torch.from_numpy(np.ascontiguousarray(elnod.reshape(-1))).to(dev)
    t_off = torch.from_numpy(off).to(dev)
    t_cnt = torch.from_numpy(cnt).to(dev)
    t_nodel = torch.from_numpy(nodel).to(dev)
    out = torch.full((nn,), float("nan"), dtype=torch.float64, device=dev)
    if stream is None:
        st = wf.lib().wf_nodal_volumes_noalloc(xyz.data_ptr(), el.data_ptr(), nn, ne, npe,
                                               t_off.data_ptr(), t_cnt.data_ptr(),
                                               t_nodel.data_ptr(), out.data_ptr(),
                                               torch.cuda.current_stream(dev).cuda_stream)
        assert st == 0, wf.STATUS.get(st, st)
        torch.cuda.synchronize(dev)
        return out.cpu().numpy()
    # on the caller's own stream: the inputs were made on the current stream,
    # so the side stream waits for it; only that stream is synchronised after
    stream.wait_stream(torch.cuda.current_stream(dev))
    st = wf.lib().wf_nodal_volumes_noalloc(xyz.data_ptr(), el.data_ptr(), nn, ne, npe,
                                           t_off.data_ptr(), t_cnt.data_ptr(),
                                           t_nodel.data_ptr(), out.data_ptr(),
                                           stream.cuda_stream)
    assert st == 0, wf.STATUS.get(st, st)
    stream.synchronize()
    return out.cpu().numpy()


def rel_err(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_noalloc_matches_domain_path_on_two_calls_in_a_row():
    torch = pytest.importorskip("torch")
    first = W.config(1, scale=(6, 5, 7))    # perturbed tetrahedra
    second = W.config(2, scale=(10, 9, 8))  # perturbed hexahedra
    d1, ref1 = domain_voln(first)
    got1 = noalloc_voln(torch, first, d1)
    assert rel_err(got1, ref1) <= TOL
    d2, ref2 = domain_voln(second)
    got2 = noalloc_voln(torch, second, d2)
    assert rel_err(got2, ref2) <= TOL
    again = noalloc_voln(torch, second, d2)
    np.testing.assert_array_equal(again, got2)
    # queued on a non-default stream of the caller: same bits
    side = torch.cuda.Stream(device=torch.device("cuda:0"))
    on_side = noalloc_voln(torch, second, d2, stream=side)
    np.testing.assert_array_equal(on_side, got2)


def test_noalloc_rejects_too_many_elements():
    L = wf.lib()
    # sizes are checked before any pointer is used (all pointers dummy, non-null)
    st = L.wf_nodal_volumes_noalloc(8, 8, 8, 1048577, 8, 8, 8, 8, 8, None)
    assert st == 5   # WF_ERR_UNSUPPORTED
    assert L.wf_nodal_volumes_noalloc(None, 8, 8, 8, 8, 8, 8, 8, 8, None) == 1
    # invalid element type and empty meshes: WF_ERR_ARG before any pointer is used
    assert L.wf_nodal_volumes_noalloc(8, 8, 8, 8, 6, 8, 8, 8, 8, None) == 1
    assert L.wf_nodal_volumes_noalloc(8, 8, 8, 0, 8, 8, 8, 8, 8, None) == 1
    assert L.wf_nodal_volumes_noalloc(8, 8, 0, 8, 8, 8, 8, 8, 8, None) == 1
