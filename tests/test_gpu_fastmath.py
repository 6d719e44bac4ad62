"""The chemistry kernels' table-driven exp and log (hyperflow_gb300/csrc/hf_fastmath.cuh)
on the GPU against numpy's libm: within 2 ulp over the fast ranges (exp |x| < 700; log
for x in [2^-1021, 2^1023), with an absolute floor of 3e-16 near x = 1 where log x
itself goes to zero), the paired form exp(x), exp(-x) likewise, and the library
results outside the fast ranges."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def evaluate(lib, x):
    xd = torch.from_numpy(x).cuda()
    outs = [torch.empty_like(xd) for _ in range(4)]
    assert lib.hf_fastmath_eval(xd.data_ptr(), xd.numel(), *[o.data_ptr() for o in outs], None) == 0
    torch.cuda.synchronize()
    return [o.cpu().numpy() for o in outs]


def ulps(got, ref):
    return np.abs(got - ref) / np.spacing(np.abs(ref))


def test_exp_and_pair_within_two_ulp(gpu):
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(-699.9, 699.9, 200000), rng.uniform(-1, 1, 100000), rng.uniform(-1e-3, 1e-3, 50000),
                        rng.uniform(-300, 20, 100000), np.arange(-64, 65) * np.log(2) / 64, [0.0, -0.0]])
    e, ep, em, _ = evaluate(gpu.lib, x)
    assert ulps(e, np.exp(x)).max() <= 2.0
    assert ulps(ep, np.exp(x)).max() <= 2.0
    assert ulps(em, np.exp(-x)).max() <= 2.0


def test_log_within_two_ulp(gpu):
    rng = np.random.default_rng(6)
    x = np.concatenate([np.exp(rng.uniform(-700, 700, 200000)), rng.uniform(150, 6000, 100000),
                        rng.uniform(0.5, 2.0, 100000), 2.0 ** np.arange(-1021, 1023, dtype=np.float64)])
    _, _, _, l = evaluate(gpu.lib, x)
    ref = np.log(x)
    err = np.abs(l - ref)
    assert np.all(err <= np.maximum(2.0 * np.spacing(np.abs(ref)), 3e-16))
    far = np.abs(ref) > 0.5
    assert ulps(l[far], ref[far]).max() <= 2.0


def test_library_outside_fast_ranges(gpu):
    x = np.array([700.0, 709.7, 710.0, -700.0, -745.0, -800.0, np.inf, -np.inf, np.nan, 1e-310, 0.0, -1.0, 2.0 ** 1023,
                  1.7e308])
    e, ep, em, l = evaluate(gpu.lib, x)
    with np.errstate(all="ignore"):
        for got, ref in ((e, np.exp(x)), (ep, np.exp(x)), (em, np.exp(-x))):
            fin = np.isfinite(ref) & (ref != 0)
            assert np.array_equal(np.isnan(got), np.isnan(ref))
            assert np.all(got[np.isinf(ref)] == ref[np.isinf(ref)])
            assert ulps(got[fin], ref[fin]).max() <= 2.0
        ref = np.log(x)
        assert np.array_equal(np.isnan(l), np.isnan(ref))
        fin = np.isfinite(ref)
        assert np.all(l[~fin & ~np.isnan(ref)] == ref[~fin & ~np.isnan(ref)])
        assert ulps(l[fin], ref[fin]).max() <= 2.0
