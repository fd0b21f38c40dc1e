"""GB300-native GP posterior + Monte-Carlo acquisition path of BoTorch.

Drop-in classes for the reference's ``SingleTaskGP.posterior``,
``qExpectedImprovement`` and ``qLogNoisyExpectedImprovement`` (value and
gradient), computed by hand-written sm_103a CUDA kernels behind the C ABI in
``include/botorch_gb300.h``.
"""

from botorch_gb300.acquisition import (qExpectedImprovement, qLogNoisyExpectedImprovement,
                                       prune_inferior_points)
from botorch_gb300.exceptions import BotorchWarning, NanError, NotPSDError, UnsupportedError
from botorch_gb300.gp_regression import GPyTorchPosterior, SingleTaskGP, Standardize
from botorch_gb300.kernels import (ConstantMean, GammaPrior, GaussianLikelihood, LogNormalPrior,
                                   MaternKernel, RBFKernel, ScaleKernel)
from botorch_gb300.sampling import SobolQMCNormalSampler, draw_sobol_normal_samples

__all__ = [
    "SingleTaskGP", "GPyTorchPosterior", "Standardize", "qExpectedImprovement",
    "qLogNoisyExpectedImprovement", "prune_inferior_points", "SobolQMCNormalSampler",
    "draw_sobol_normal_samples", "MaternKernel", "RBFKernel", "ScaleKernel", "GaussianLikelihood",
    "ConstantMean", "NotPSDError", "NanError", "UnsupportedError", "BotorchWarning",
    "LogNormalPrior", "GammaPrior",
]
