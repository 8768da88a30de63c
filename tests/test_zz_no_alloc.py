"""The allocation-free entry point nb_reduce_fp64_static.

Some callers cannot allocate device memory: a serving process whose device memory all belongs
to a pre-sized pool, or code that must not call cudaMalloc while another thread is capturing
work into a CUDA graph.  For them the library keeps the scratch of its FP64 conservation
totals (per-block partial sums) in a static device array, and the entry point takes only the
input planes and a device output.  This test checks, through the C ABI, that two calls in a row
give the totals of the handle-based nb_reduce_fp64 (which allocates its scratch at nb_create),
and that a size beyond the array's limit is refused.  Collected last (file name) so that a run
stopping at its first failure has already run every other test.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _lib():
    from nebulaviewer_gb300 import build
    build.build(verbose=False)
    from nebulaviewer_gb300 import _lib as L
    return L


def test_static_totals_match_handle_totals_twice():
    L = _lib()
    lib = L.load()
    from nebulaviewer_gb300.sim import Sim
    assert torch.cuda.is_available()
    stream = torch.cuda.current_stream()
    # two calls in a row per shape, different inputs: 161 x 128 x 96 = 1,978,368 cells = 30 full
    # blocks of 65536 cells and a partial one of 12,288; 7 x 9 x 12 = 756 cells, one partial block
    for shape, seed in (((161, 128, 96), 11), ((161, 128, 96), 12), ((7, 9, 12), 13), ((7, 9, 12), 14)):
        n = int(np.prod(shape))
        g = torch.Generator(device="cuda").manual_seed(seed)
        rho = torch.rand(shape, device="cuda", generator=g) * 10 + 0.01
        mom = [torch.randn(shape, device="cuda", generator=g) for _ in range(3)]
        sim = Sim.from_state(shape, 1.0 / 128, rho, [], [], [], [], {}, mom=mom, rays=(8, 16), fuv_grid=(4, 4, 8),
                             start_main=False)
        ref = np.array(sim.conservation()) / sim.dx ** 3          # handle-based nb_reduce_fp64 (raw sums)
        out = torch.full((4,), float("nan"), dtype=torch.float64, device="cuda")
        rc = lib.nb_reduce_fp64_static(sim._rho.data_ptr(), sim._mx.data_ptr(), sim._my.data_ptr(),
                                       sim._mz.data_ptr(), n, out.data_ptr(), stream.cuda_stream)
        assert rc == 0, lib.nb_static_last_error()
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        exact = np.array([t.double().sum().item() for t in (sim._rho, sim._mx, sim._my, sim._mz)])
        # different block partitions sum in a different order: FP64 rounding only
        assert np.allclose(got, ref, rtol=1e-12, atol=1e-9 * np.abs(exact).max()), (got, ref)
        assert np.allclose(got, exact, rtol=1e-12, atol=1e-9 * np.abs(exact).max())
        sim.close()


def test_static_totals_refuse_sizes_beyond_the_array():
    L = _lib()
    lib = L.load()
    x = torch.zeros(4, device="cuda")
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    p = x.data_ptr()
    rc = lib.nb_reduce_fp64_static(p, p, p, p, (1 << 30) + 1, out.data_ptr(), None)
    assert rc == -4                                            # NB_ERR_LIMIT, before any device work
    assert b"2^30" in lib.nb_static_last_error()
