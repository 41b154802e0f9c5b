"""g6x_force_dev_noalloc: the force entry point that allocates no device
memory (for callers whose device memory is owned by a host framework, or
whose step loop cannot absorb cudaMalloc's synchronisation).  Its split-j
partial sums live in a fixed 16 MiB array inside the library.

Checked through the C ABI against g6x_force_dev (the allocating entry point)
on the same inputs, twice in a row (the shared array keeps the previous
call's contents), in both precisions and with and without the nearest
neighbour: the launch shape and the fixed-order merge are the same, so the
results must be bit-identical.  This file is collected last so that a run
stopping at the first failure has already run every other test."""
import numpy as np
import pytest

import amuse_gb300 as ag
from amuse_gb300 import ic

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("want_nn", [True, False], ids=["nn", "no-nn"])
@pytest.mark.parametrize("prec", [ag.SPLIT, ag.FP64], ids=["split", "fp64"])
def test_noalloc_matches_allocating_entry_point(g6, prec, want_nn):
    torch = pytest.importorskip("torch")
    g6.set_precision(prec)
    try:
        np.random.seed(31)
        nj = 20000
        m, x, v = ic.plummer(nj)
        g6.load_particles(m, x, v)
        outs = []
        for seed, ni in ((1, 1000), (2, 1000)):  # two calls in a row, new inputs each time
            rng = np.random.RandomState(seed)
            sel = np.sort(rng.choice(nj, ni, replace=False)).astype(np.int32)
            dx = torch.tensor(x[sel], device="cuda").contiguous()
            dv = torch.tensor(v[sel], device="cuda").contiguous()
            ds = torch.tensor(sel, device="cuda")
            res = {}
            for name in ("alloc", "noalloc"):
                da = torch.full((ni, 3), float("nan"), dtype=torch.float64, device="cuda")
                dj = torch.full_like(da, float("nan"))
                dp = torch.full((ni,), float("nan"), dtype=torch.float64, device="cuda")
                dn = torch.full((ni,), -7, dtype=torch.int32, device="cuda") if want_nn else None
                torch.cuda.synchronize()
                f = g6.force_dev if name == "alloc" else g6.force_dev_noalloc
                f(0.0, 1e-4, nj, ni, dx.data_ptr(), dv.data_ptr(), ds.data_ptr(), da.data_ptr(),
                  dj.data_ptr(), dp.data_ptr(), dn.data_ptr() if want_nn else None, sync=True)
                res[name] = dict(acc=da.cpu().numpy(), jerk=dj.cpu().numpy(),
                                 pot=dp.cpu().numpy())
                if want_nn:
                    res[name]["nn"] = dn.cpu().numpy()
            # the scratch array is actually used: this shape splits j across CTAs
            assert g6.stats()["nsplit"] > 1
            a, b = res["alloc"], res["noalloc"]
            assert np.all(np.isfinite(b["acc"])) and np.all(np.isfinite(b["pot"]))
            for k in a:
                assert np.array_equal(b[k], a[k]), k
            if want_nn:
                assert np.all(b["nn"] >= 0)
            outs.append(b)
        assert not np.array_equal(outs[0]["pot"], outs[1]["pot"])
    finally:
        g6.set_precision(ag.SPLIT)


def test_noalloc_refuses_oversized_scratch(g6):
    torch = pytest.importorskip("torch")
    g6.set_precision(ag.SPLIT)
    np.random.seed(32)
    n = 131072
    m, x, v = ic.plummer(n)
    g6.load_particles(m, x, v)
    dx = torch.tensor(x, device="cuda").contiguous()
    dv = torch.tensor(v, device="cuda").contiguous()
    da = torch.empty((n, 3), dtype=torch.float64, device="cuda")
    dj = torch.empty_like(da)
    dp = torch.empty(n, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    # all 131072 i against 131072 j splits j 13 ways: ~100 MB of partials
    with pytest.raises(ag.G6Error, match="scratch"):
        g6.force_dev_noalloc(0.0, 1e-6, n, n, dx.data_ptr(), dv.data_ptr(), None, da.data_ptr(),
                             dj.data_ptr(), dp.data_ptr(), None, sync=True)
