"""lg_diffuse_noalloc: the diffusion entry point for callers that cannot
allocate device memory (their memory belongs to another allocator or a fixed
arena). It must give lg_diffuse's result from caller-owned device buffers,
using only the library's fixed scratch array, on consecutive calls.

This file is collected last (tests/test_zz_*) so that a run stopping at the
first failure has already run every other test; it also passes alone."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_noalloc_diffuse_matches_lg_diffuse():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from lightgraph_gb300 import Context, _capi, scenes

    sc = scenes.small(n_points=700, width=16, height=16)
    ctx = Context(0)
    try:
        scenes.load_into(ctx, sc)
        ctx.build_graphs(sc.points, sc.radius_sq, sc.max_connect)
        ctx.march_edges()
        dist = ctx.solve_paths(want=True)[0]  # n x n, diagonal 0
        L = ctx.vertex_light(want=True)
        D_ref = ctx.diffuse(want=True)  # the existing entry point
        lib = ctx.lib
        n = dist.shape[0]
        ld = n + 4  # any leading dimension >= n
        S_dev = torch.full((n, ld), float("inf"), device="cuda", dtype=torch.float32)
        S_dev[:, :n] = torch.from_numpy(dist).cuda()
        L_dev = torch.from_numpy(np.ascontiguousarray(L)).cuda()
        D_dev = torch.empty((n, 3), device="cuda", dtype=torch.float32)
        ext = (C.c_double * 3)(*sc.shader.getExtinction())
        stream = torch.cuda.current_stream().cuda_stream
        # the FP64 oracle's diffusion of the same solved paths and radiance
        from oracle import pyoracle as po
        a = -np.array(sc.shader.getExtinction())
        T = np.exp(-a[None, None, :] * dist.astype(np.float64)[:, :, None])
        idx = np.arange(n)
        T[idx, idx, :] = 1.0
        D_oracle = po.diffuse(T, L.astype(np.float64))
        for _ in range(2):  # the first call sets up the scratch address, the second reuses it
            D_dev.fill_(float("nan"))
            st = lib.lg_diffuse_noalloc(S_dev.data_ptr(), n, ld, L_dev.data_ptr(), D_dev.data_ptr(), ext, stream)
            assert st == _capi.LG_OK
            torch.cuda.synchronize()
            got = D_dev.cpu().numpy()
            # the same kernels in the same order as lg_diffuse: the same bits
            assert np.array_equal(got, D_ref)
            assert np.allclose(got, D_oracle, rtol=1e-4, atol=1e-6)
        # sizes beyond the fixed scratch array (LG_NOALLOC_MAX_POINTS = 8192) are
        # refused, with no work enqueued
        big = 8193
        st = lib.lg_diffuse_noalloc(S_dev.data_ptr(), big, big, L_dev.data_ptr(), D_dev.data_ptr(), ext, stream)
        assert st == _capi.LG_ERR_INVALID
    finally:
        ctx.close()
