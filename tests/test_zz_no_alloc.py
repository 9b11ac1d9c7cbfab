"""The allocation-free compaction entry point (grt_compact_hits_static) against the regular
one (grt_compact_hits).

grt_compact_hits_static serves callers that cannot call cudaMalloc: renderers whose device
memory all comes from their own up-front pool, and frame loops that cannot take cudaMalloc's
implicit device synchronisation. It keeps its tile counts in a fixed device array shared by all
calls, so this test makes two calls in a row (the second smaller, over different hits) and
checks each against the regular entry point, which takes its scratch from a context; then an
empty call, which must still set the count to zero. The file is named so that pytest collects
it last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRT_OK, GRT_ERR_TOO_LARGE = 0, 10
MAX_HITS = 33554432


@pytest.fixture(autouse=True)
def _needs_cuda():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _random_hits(n, seed, hit_fraction):
    import torch
    g = np.random.default_rng(seed)
    h = np.zeros((n, 4), np.float32)
    valid = g.random(n) < hit_fraction
    h[:, 0] = np.where(valid, g.random(n).astype(np.float32) * 10, np.float32(3.4028234663852886e38))
    return torch.from_numpy(h).cuda(), np.nonzero(valid)[0]


def test_static_compaction_matches_context_compaction(api):
    import torch
    lib = api.lib()
    fn = lib.grt_compact_hits_static
    fn.restype = ctypes.c_int
    fn.argtypes = [ctypes.c_void_p, ctypes.c_uint32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
    rt = api.BatchRayTracer(0)
    stream = torch.cuda.current_stream().cuda_stream
    try:
        for n, seed, frac in [(5_000_000, 1, 0.37), (1_000_003, 2, 0.81)]:
            hits, want = _random_hits(n, seed, frac)
            idx_static = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            cnt_static = torch.full((1,), -1, dtype=torch.int32, device="cuda")
            idx_ctx = torch.full((n,), -1, dtype=torch.int32, device="cuda")
            cnt_ctx = torch.full((1,), -1, dtype=torch.int32, device="cuda")
            assert fn(hits.data_ptr(), n, idx_static.data_ptr(), cnt_static.data_ptr(), stream) == GRT_OK
            rt.compact_hits(hits, idx_ctx, cnt_ctx, stream)
            torch.cuda.synchronize()
            c = int(cnt_static.item())
            assert c == int(cnt_ctx.item()) == want.size
            assert torch.equal(idx_static[:c], idx_ctx[:c])
            assert (idx_static[:c].cpu().numpy() == want).all()
        # no hits at all: the count is written (zero) and no kernel reads the array
        cnt_static.fill_(-1)
        assert fn(hits.data_ptr(), 0, idx_static.data_ptr(), cnt_static.data_ptr(), stream) == GRT_OK
        torch.cuda.synchronize()
        assert int(cnt_static.item()) == 0
        # beyond the fixed capacity the call is refused before anything runs
        assert fn(hits.data_ptr(), MAX_HITS + 1, idx_static.data_ptr(), cnt_static.data_ptr(), stream) == \
            GRT_ERR_TOO_LARGE
    finally:
        rt.close()
