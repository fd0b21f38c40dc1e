"""The oracle against golden vectors produced by the reference's own modules."""

from pathlib import Path

import numpy as np
import pytest
import torch

from oracle import safe_math
from oracle.sampling import draw_sobol_normal_samples

GOLD = np.load(Path(__file__).resolve().parent / "golden" / "reference_golden.npz")


def t(name):
    return torch.from_numpy(GOLD[name])


def close(a, b, rtol=1e-15, atol=0.0):
    a = a.numpy() if isinstance(a, torch.Tensor) else a
    np.testing.assert_allclose(a, b, rtol=rtol, atol=atol)


def test_cauchy_fatplus():
    x = t("x")
    close(safe_math.cauchy(x), GOLD["cauchy"])
    close(safe_math.fatplus(x, 1.0), GOLD["fatplus_tau1"])
    close(safe_math.log_fatplus(x, 1.0), GOLD["log_fatplus_tau1"])
    close(safe_math.log_fatplus(t("x_small"), 1e-6), GOLD["log_fatplus_tau1e-6"])


def test_pareto():
    close(safe_math.pareto(t("x_pareto"), 2.0), GOLD["pareto2"])


@pytest.mark.parametrize("tau", ["1e-2", "1"])
def test_fatmax_with_infinities(tau):
    out = safe_math.fatmax(t("fatmax_in"), dim=-1, tau=float(tau))
    close(out, GOLD[f"fatmax_tau{tau}"])


def test_logmeanexp_logsumexp():
    close(safe_math.logmeanexp(t("lme_in"), dim=0), GOLD["logmeanexp"])
    close(safe_math.logsumexp(t("lme_in"), dim=0), GOLD["logsumexp"])


def test_qlognei_utility_and_reduction():
    Y, bf = t("qlognei_Y"), t("qlognei_best_f")
    li = safe_math.log_fatplus(Y - bf[:, None, None], 1e-6)
    close(li, GOLD["qlognei_li"])
    v = safe_math.logmeanexp(safe_math.fatmax(li, dim=-1, tau=1e-2), dim=0)
    close(v, GOLD["qlognei_value"])


@pytest.mark.parametrize("d,n,seed", [(4, 256, 0), (6, 256, 0), (10, 512, 0), (12, 512, 0),
                                      (2, 16, 12345), (22, 64, 7)])
def test_sobol_normal_bit_exact(d, n, seed):
    z = draw_sobol_normal_samples(d, n, seed)
    assert np.array_equal(z.numpy(), GOLD[f"sobol_normal_d{d}_n{n}_s{seed}"])


def test_product_sampler_bit_exact():
    from botorch_gb300.sampling import draw_sobol_normal_samples as product_draw

    for d, n, seed in ((4, 256, 0), (12, 512, 0), (22, 64, 7)):
        assert np.array_equal(product_draw(d, n, seed).numpy(), GOLD[f"sobol_normal_d{d}_n{n}_s{seed}"])
