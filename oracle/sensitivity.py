"""ORACLE (test infrastructure): how much the float64 qLogNEI value and gradient of each
t-batch move when the posterior mean of its q points moves by a small amount.

The mixed-precision GPU path forms the posterior mean from float32 kernel values and
float16-split cross-covariance products; its mean carries an error of about 1e-6 in
standardised units (float32 rounding of the kernel values times the cancellation in
K(x, Xt) (K + s2 I)^-1 (y - m)). For a t-batch whose dominant MC samples sit close to
the incumbent (improvements small against |mean|), log_fatplus and the smooth maxima
amplify that error (by up to 1 / |u| for an improvement u, by 1 / tau_relu near zero),
so no float32 posterior reproduces its gradient to 1e-4. This module measures that
amplification on the oracle itself: the relative change of the value and of the
gradient under a shift ``delta`` of the standardised mean of the q points, uniform
(+delta on every point) and alternating (+delta, -delta, ...), the larger of the two.
Tests bound the mixed path per t-batch by max(bar, c x sensitivity).
"""

from __future__ import annotations

import torch

MEAN_DELTA = 1e-6  # standardised units: the float32 error of the mixed path's posterior mean


def mean_sensitivity(acqf, X: torch.Tensor, value: torch.Tensor, grad: torch.Tensor,
                     delta: float = MEAN_DELTA) -> tuple[torch.Tensor, torch.Tensor]:
    """Per t-batch relative change of value and gradient of the oracle ``acqf``
    (QLogNoisyExpectedImprovement) under the mean shifts; ``value`` / ``grad`` are
    its unperturbed outputs at X (b x q x d)."""
    q = X.shape[-2]
    model = acqf.model
    sv = torch.zeros(X.shape[0], dtype=torch.float64)
    sg = torch.zeros(X.shape[0], dtype=torch.float64)
    alt = torch.tensor([1.0 if i % 2 == 0 else -1.0 for i in range(q)], dtype=torch.float64)
    try:
        for shift in (torch.full((q,), delta, dtype=torch.float64), delta * alt):
            model.mean_shift = shift
            v, g = acqf.value_and_grad(X)
            sv = torch.maximum(sv, (v - value).abs() / value.abs())
            sg = torch.maximum(sg, (g - grad).flatten(1).norm(dim=1) / grad.flatten(1).norm(dim=1))
    finally:
        model.mean_shift = None
    return sv, sg
