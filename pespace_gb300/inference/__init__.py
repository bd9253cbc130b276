"""Likelihoods (single-sample plugin path and the batched plan engine)."""

from .likelihood import (  # noqa: F401
    CapturedStep,
    LikelihoodBilbyInterface,
    WhittleLikelihood,
    WhittleLikelihoodCuda,
    compute_whittle_likelihood,
    compute_whittle_likelihood_ti,
    log_likelihood,
    noise_weighted_inner_product,
)
from .fisher import fisher_matrix, sample_from_fisher, wrap_angle_params  # noqa: F401,E402
