"""hdc_search_plain_noalloc: the plain top-k search for callers that are not
allowed to allocate device memory (a host that owns every device buffer
through its own pool, a fully reserved memory budget, or a loop that cannot
pay for the synchronisation of cudaMalloc / cudaFree).  Its scratch is a
fixed array inside the library, so it is checked here, through the C ABI,
against the allocating entry point hdc_search_plain on the same inputs, on
two calls in a row with different inputs (the second call must not see the
first call's leftovers).  Results must be identical: indices, dots, float
scores and FP64 cosines.

This file is collected last on purpose, so that a run that stops at the
first failure has run every other test before this one."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _inputs(torch, dev, seed, nq, nr, dim, vmax):
    g = np.random.default_rng(seed)
    q = torch.from_numpy(g.integers(-vmax, vmax + 1, (nq, dim)).astype(np.int16)).to(dev)
    r = torch.from_numpy(g.integers(-vmax, vmax + 1, (nr, dim)).astype(np.int16)).to(dev)
    r[7] = r[2]  # a tie, broken by the lower index
    return q, r


def _noalloc(hdc, torch, ctx, q, qn, mq, r, rn, mr, k, mode):
    nq = q.shape[0]
    out = (torch.full((nq, k), 7.0, dtype=torch.float32, device=q.device),
           torch.full((nq, k), -7, dtype=torch.int32, device=q.device),
           torch.full((nq, k), 7.0, dtype=torch.float64, device=q.device),
           torch.full((nq, k), -7, dtype=torch.int64, device=q.device))
    p = hdc.ptr
    st = hdc.lib().hdc_search_plain_noalloc(ctx.h, p(q), p(qn), nq, mq, p(r), p(rn), r.shape[0], mr, k, mode,
                                            p(out[0]), p(out[1]), p(out[2]), p(out[3]), hdc.stream_ptr())
    hdc.check(st)
    return out


def test_noalloc_matches_allocating_search_twice(hdc, cuda):
    import torch
    dim, k, mode = 1024, 5, hdc.SCORE_NORM
    ctx = hdc.Context(dim, 8, 150, 10)
    for call, (seed, nq, nr) in enumerate([(21, 300, 2000), (22, 170, 3100)]):
        q, r = _inputs(torch, cuda, seed, nq, nr, dim, 300)
        mq = torch.zeros(1, dtype=torch.int32, device=cuda)
        mr = torch.zeros(1, dtype=torch.int32, device=cuda)
        qn, rn = ctx.norms(q, mq), ctx.norms(r, mr)
        torch.cuda.synchronize()
        mq, mr = int(mq.item()), int(mr.item())
        want = ctx.search_plain(q, qn, mq, r, rn, mr, k, mode)
        got = _noalloc(hdc, torch, ctx, q, qn, mq, r, rn, mr, k, mode)
        torch.cuda.synchronize()
        for w, g in zip(want, got):
            assert torch.equal(w, g), "call %d differs from hdc_search_plain" % call


def test_noalloc_rejects_batches_beyond_the_fixed_scratch(hdc, cuda):
    import torch
    dim, k = 64, 32
    ctx = hdc.Context(dim, 8, 150, 10)
    nq = 65536  # 65536 queries x 32 results x 16 bytes = 32 MiB of lists > 16 MiB
    q = torch.zeros((nq, dim), dtype=torch.int16, device=cuda)
    r = torch.ones((64, dim), dtype=torch.int16, device=cuda)
    qn, rn = ctx.norms(q), ctx.norms(r)
    need = ctx.workspace_bytes(nq, 64, k)
    assert need > hdc.lib().hdc_search_workspace_bytes(ctx.h, 1, 64, k)
    with pytest.raises(hdc.HDCError) as e:
        _noalloc(hdc, torch, ctx, q, qn, 1, r, rn, 1, k, hdc.SCORE_NORM)
    assert e.value.status == 2
    assert "scratch" in str(e.value)


def test_noalloc_checks_k_before_the_scratch_size(hdc, cuda):
    """k = 33 is an invalid argument (as for hdc_search_plain) even on a batch
    whose lists would not fit the fixed scratch; k above nr is clamped to nr."""
    import torch
    dim = 64
    ctx = hdc.Context(dim, 8, 150, 10)
    nq = 65536
    q = torch.ones((nq, dim), dtype=torch.int16, device=cuda)
    r = torch.ones((64, dim), dtype=torch.int16, device=cuda)
    qn, rn = ctx.norms(q), ctx.norms(r)
    p = hdc.ptr
    out = [torch.empty((nq, 32), dtype=t, device=cuda) for t in (torch.float32, torch.int32, torch.float64,
                                                                 torch.int64)]
    for fn in ("hdc_search_plain_noalloc", "hdc_search_plain"):
        extra = [] if fn.endswith("noalloc") else [None, 0]
        st = getattr(hdc.lib(), fn)(ctx.h, p(q), p(qn), nq, 1, p(r), p(rn), 64, 1, 33, hdc.SCORE_NORM,
                                    *[p(o) for o in out], *extra, hdc.stream_ptr())
        assert st == 1 and b"k must be in 1..32" in hdc.lib().hdc_last_error(), fn
    # 40 > nr = 4 is clamped to 4 (a small batch: fits the scratch)
    q4, r4 = q[:8], r[:4]
    got = _noalloc(hdc, torch, ctx, q4, qn[:8], 1, r4, rn[:4], 1, 4, hdc.SCORE_NORM)
    st = hdc.lib().hdc_search_plain_noalloc(ctx.h, p(q4), p(qn), 8, 1, p(r4), p(rn), 4, 1, 40, hdc.SCORE_NORM,
                                            p(got[0]), p(got[1]), p(got[2]), p(got[3]), hdc.stream_ptr())
    assert st == 0
    torch.cuda.synchronize()
    assert torch.equal(got[1][:, :4].cpu(), torch.arange(4, dtype=torch.int32).expand(8, 4))
