"""kgb_population_noalloc against kgb_population, through the C ABI.

The allocation-free entry point serves callers that cannot allocate device
memory when they need the particle count (frameworks that own all device
memory through their own pool, latency-bound loops).  It must give the same FP64
population as the context-based kgb_population, within the 1e-12 relative
tolerance of the other FP64 parity tests, on two calls in a row (the second
call reuses the static scratch the first one left behind), and from a CUDA
graph that captured the call, on every replay.  This file sorts last so that
a run stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_population_noalloc_matches_population():
    import torch
    from kripke_gb300 import abi

    lib = abi.load()
    ctx = abi.Context(0)
    ctx.generate(zones=(12, 10, 8), groups=8, quad=(4, 8), legendre=2, scatter=1, geometry=1, gset=1, dset=8,
                 layout="DGZ")
    ctx.solve(2)
    want = ctx.population()

    # the same psi in the device nesting [zone][group][direction]
    Z, G, D, Ds = 12 * 10 * 8, 8, 32, 4
    psi = ctx.download("psi").reshape(8, Ds, G, Z)          # DGZ chunks: one per octant, [d][g][z]
    psi_dev = np.ascontiguousarray(psi.transpose(3, 2, 0, 1).reshape(Z, G, D))
    dev = torch.device("cuda", 0)
    t_psi = torch.from_numpy(psi_dev).to(dev)
    t_w = torch.from_numpy(ctx.download("quadrature/w")).to(dev)
    t_vol = torch.from_numpy(ctx.download("volume")).to(dev)
    t_out = torch.full((2,), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    err = ctypes.create_string_buffer(256)

    results = []
    for call in range(2):
        rc = lib.kgb_population_noalloc(t_psi.data_ptr(), t_w.data_ptr(), t_vol.data_ptr(), Z, G, D,
                                        t_out.data_ptr() + 8 * call, stream, err, len(err))
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize(dev)
        results.append(float(t_out[call].item()))
    for got in results:
        assert got == pytest.approx(want, rel=1e-12)
    assert results[0] == results[1]  # fixed summation order: bitwise repeatable

    # captured into a CUDA graph after the calls above (which looked up the scratch address):
    # every replay runs both launches again and rewrites the static scratch, bit for bit
    t_cap = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    side = torch.cuda.Stream(dev)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=side):
        rc = lib.kgb_population_noalloc(t_psi.data_ptr(), t_w.data_ptr(), t_vol.data_ptr(), Z, G, D,
                                        t_cap.data_ptr(), side.cuda_stream, err, len(err))
    assert rc == 0, err.value.decode()
    for _ in range(2):
        t_cap.fill_(-1.0)
        graph.replay()
        torch.cuda.synchronize(dev)
        assert float(t_cap.item()) == results[0]

    # sizes beyond the static scratch are rejected before any launch
    rc = lib.kgb_population_noalloc(t_psi.data_ptr(), t_w.data_ptr(), t_vol.data_ptr(), 1 << 40, G, D,
                                    t_out.data_ptr(), stream, err, len(err))
    assert rc == 1 and b"exceeds" in err.value
    ctx.close()
