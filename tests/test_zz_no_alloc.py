"""The allocation-free pair-list entry point (nd_leaf_pairs_noalloc_dev).

Some callers cannot call cudaMalloc -- code living under a runtime that owns
the device memory pool, or loops where an allocation would stall the device.
For them the library runs the pair-list pipeline on a fixed device array.  This
test calls that entry point through the C ABI twice in a row (the second call
re-uses the array the first one left behind) and checks each result against the
allocating entry point nd_leaf_pairs_dev: same count and the same pairs in the
same order, bit for bit (the tolerance for index work).  It also checks that a
request above the stated limit is refused.  The file is named to be collected
last.
"""
import ctypes

import numpy as np
import pytest

from helpers import uniform

pytestmark = pytest.mark.gpu

ND_ERR_ARG = -1


def _noalloc(L, xt, cs, order, mode, pi, pj, pd, cap, stream):
    count = ctypes.c_int64()
    st = L.nd_leaf_pairs_noalloc_dev(xt.data_ptr(), ctypes.byref(cs), order, mode,
                                     pi.data_ptr() if pi is not None else None,
                                     pj.data_ptr() if pj is not None else None,
                                     pd.data_ptr() if pd is not None else None,
                                     cap, ctypes.byref(count), stream)
    return st, count.value


def test_no_alloc_matches_allocating_entry_point(nd):
    import torch
    from naivedynamics import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    cases = [(101, 4096, 0.12, nd.ND_ORDER_REFERENCE, nd.ND_PAIRS_ORDERED),
             (102, 8000, 0.09, nd.ND_ORDER_SPATIAL, nd.ND_PAIRS_ORDERED)]
    for seed, n, r, order, mode in cases:
        x = uniform(seed, n)
        xt = torch.from_numpy(x).cuda()
        spec = nd.SpheresBVHSpecs(r, n, 4)
        cs = spec.c_spec()
        dummy = torch.empty(1, dtype=torch.int32, device="cuda")
        st, cnt = nd.neighbor_pairs_dev(xt, spec, dummy, dummy, dummy.float(), 0, order=order,
                                        mode=mode)
        assert cnt > 0
        ref = [torch.empty(cnt, dtype=torch.int32, device="cuda") for _ in range(2)]
        ref.append(torch.empty(cnt, dtype=torch.float32, device="cuda"))
        st, cnt_ref = nd.neighbor_pairs_dev(xt, spec, *ref, cnt, order=order, mode=mode)
        assert st == 0 and cnt_ref == cnt
        torch.cuda.synchronize()
        out = [torch.full((cnt,), -1, dtype=torch.int32, device="cuda") for _ in range(2)]
        out.append(torch.full((cnt,), -1.0, dtype=torch.float32, device="cuda"))
        torch.cuda.synchronize()
        st, c_na = _noalloc(L, xt, cs, order, mode, *out, cnt, stream)
        assert st == 0 and c_na == cnt
        torch.cuda.synchronize()
        assert torch.equal(out[0], ref[0]) and torch.equal(out[1], ref[1])
        assert torch.equal(out[2].view(torch.int32), ref[2].view(torch.int32))
        # capacity 0 only counts
        st, c0 = _noalloc(L, xt, cs, order, mode, None, None, None, 0, stream)
        assert st == _lib.ND_NEED_REALLOC and c0 == cnt


def test_no_alloc_unordered_pair_set(nd):
    # unordered mode (one-pass emission here, two-phase in the allocating
    # entry point): the same pairs, each with the same distance bits
    import torch
    from naivedynamics import _lib
    L = _lib.lib()
    stream = torch.cuda.current_stream().cuda_stream
    x = uniform(103, 16384)
    xt = torch.from_numpy(x).cuda()
    spec = nd.SpheresBVHSpecs(0.08, len(x), 4)
    dummy = torch.empty(1, dtype=torch.int32, device="cuda")
    st, cnt = nd.neighbor_pairs_dev(xt, spec, dummy, dummy, dummy.float(), 0,
                                    order=nd.ND_ORDER_SPATIAL, mode=nd.ND_PAIRS_UNORDERED)
    assert cnt > 0
    outs = []
    for noalloc in (False, True):
        o = [torch.empty(cnt, dtype=torch.int32, device="cuda") for _ in range(2)]
        o.append(torch.empty(cnt, dtype=torch.float32, device="cuda"))
        if noalloc:
            st, c = _noalloc(L, xt, spec.c_spec(), nd.ND_ORDER_SPATIAL, nd.ND_PAIRS_UNORDERED,
                             *o, cnt, stream)
        else:
            st, c = nd.neighbor_pairs_dev(xt, spec, *o, cnt, order=nd.ND_ORDER_SPATIAL,
                                          mode=nd.ND_PAIRS_UNORDERED)
        torch.cuda.synchronize()
        assert st == 0 and c == cnt
        i, j, d = (t.cpu().numpy() for t in o)
        k = np.lexsort((j, i))
        outs.append((i[k], j[k], d[k].view(np.int32)))
    for a, b in zip(*outs):
        assert np.array_equal(a, b)


def test_no_alloc_rejects_oversize(nd):
    import torch
    from naivedynamics import _lib
    L = _lib.lib()
    n = 65536 + 4
    xt = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    cs = nd.SpheresBVHSpecs(0.1, n, 4).c_spec()
    st, _ = _noalloc(L, xt, cs, 0, 0, None, None, None, 0, torch.cuda.current_stream().cuda_stream)
    assert st == ND_ERR_ARG
