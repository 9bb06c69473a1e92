"""The allocation-free entry point pf_transport_tdb_noalloc.

It exists for callers that cannot give the library a device workspace
(host codes that reserve all device memory through their own allocator and
forbid later cudaMalloc).  Its scratch is a static device array shared by
all calls, so two calls in a row must both reproduce the workspace-based
entry point pf_transport_tdb_dev on the same inputs.  This file is named so
that pytest collects it last.
"""
import ctypes as C

import numpy as np
import pytest

from phinfortran_gb300 import _abi, systems
from phinfortran_gb300.transport import BLOCK_NAMES, TdbBlocks, fortran_block

pytestmark = pytest.mark.gpu


def _device_case(torch, blocks, E):
    nq, (n, nl, nr, L), arrs = TdbBlocks.from_dict(blocks).stacked()
    dev = {k: torch.from_numpy(fortran_block(v).copy()).cuda() for k, v in arrs.items()}
    Ed = torch.from_numpy(np.ascontiguousarray(E)).cuda()
    return (n, nl, nr, L, nq), dev, Ed


def _outputs(torch, npts):
    return (torch.zeros(npts, dtype=torch.float64, device="cuda"),
            torch.zeros(npts, dtype=torch.float64, device="cuda"),
            torch.zeros(npts, dtype=torch.int32, device="cuda"),
            torch.zeros(2 * npts, dtype=torch.int32, device="cuda"))


@pytest.mark.parametrize("case", ["ribbon", "phonon_uneven_q"])
def test_noalloc_matches_workspace_entry(cuda_ready, case):
    import torch
    lib = _abi.load()
    if case == "ribbon":
        b, E, p = systems.tb_ribbon(W=32, L=60, ne=96)
        qidx = None
    else:
        b0, E0, p, _ = systems.sc_phonon(ne=64, L=6)
        b1, _, _, _ = systems.sc_phonon(ne=64, L=6, mass_range=(1.5, 2.5), seed_index=9)
        b = {k: np.stack([b0[k], b1[k]]) for k in b0}
        E = np.concatenate([E0, E0])
        qidx = np.repeat(np.arange(2, dtype=np.int32), E0.size)
    (n, nl, nr, L, nq), dev, Ed = _device_case(torch, b, E)
    npts = E.size
    qd = None if qidx is None else torch.from_numpy(qidx).cuda()
    blk = [dev[k].data_ptr() for k in BLOCK_NAMES]
    args = (p["eta"], p["eta0"], p["dev_factor"], p["convergence"], 500, 1)
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)

    # reference: the workspace entry point
    tl0, tr0, st0, it0 = _outputs(torch, npts)
    ws = lib.pf_transport_tdb_workspace_size(n, nl, nr, nq, npts)
    work = torch.empty(ws, dtype=torch.uint8, device="cuda")
    _abi.check(lib.pf_transport_tdb_dev(n, nl, nr, L, nq, *blk, npts, Ed.data_ptr(),
                                        None if qd is None else qd.data_ptr(), None, *args,
                                        tl0.data_ptr(), tr0.data_ptr(), st0.data_ptr(), it0.data_ptr(),
                                        work.data_ptr(), work.numel(), stream))
    torch.cuda.synchronize()
    ref_l, ref_r = tl0.cpu().numpy(), tr0.cpu().numpy()
    assert (st0.cpu().numpy() == 0).all()

    # two calls in a row through the allocation-free entry point
    for _ in range(2):
        tl, tr, st, it = _outputs(torch, npts)
        _abi.check(lib.pf_transport_tdb_noalloc(n, nl, nr, L, nq, *blk, npts, Ed.data_ptr(),
                                                None if qd is None else qd.data_ptr(), None, *args,
                                                tl.data_ptr(), tr.data_ptr(), st.data_ptr(), it.data_ptr(),
                                                stream))
        torch.cuda.synchronize()
        # same kernel and arithmetic; only the number of concurrent CTAs may
        # differ, which does not change any per-point result
        np.testing.assert_allclose(tl.cpu().numpy(), ref_l, rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(tr.cpu().numpy(), ref_r, rtol=1e-12, atol=1e-14)
        assert (st.cpu().numpy() == 0).all()
        assert np.array_equal(it.cpu().numpy(), it0.cpu().numpy())


def test_noalloc_rejects_oversized_problem(cuda_ready):
    """A q count whose scratch exceeds the static maximum is refused cleanly.
    Every pointer is a real device buffer holding the blocks of q = 0, the
    one point uses q = 0 and the leads differ in size (so no lead-mirror
    pass over all q is made): a refusal that came too late would still only
    read valid memory."""
    import torch
    lib = _abi.load()
    n, nl, nr = 4, 4, 6
    nq = (64 << 20) // 4          # lead-mirror flags alone exceed the 32 MiB array
    sizes = [nl * nl, nl * nl, nr * nr, nr * nr, n * n, 0, nl * n, nr * n]
    blocks = [torch.zeros(2 * max(s, 1), dtype=torch.float64, device="cuda") for s in sizes]
    E = torch.ones(1, dtype=torch.float64, device="cuda")
    tl = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    qidx = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = lib.pf_transport_tdb_noalloc(n, nl, nr, 1, nq, *[b.data_ptr() for b in blocks], 1, E.data_ptr(),
                                      qidx.data_ptr(), None, 0.0, 1e-6, 1.0, 1e-14, 10, 0, tl.data_ptr(), None,
                                      st.data_ptr(), None, None)
    torch.cuda.synchronize()
    assert rc == -3
    assert b"static maximum" in lib.pf_last_error()
