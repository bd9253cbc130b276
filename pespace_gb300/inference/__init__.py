"""Likelihoods (single-sample plugin path and the batched plan engine)."""

from .likelihood import (  # noqa: F401
    CapturedStep,
    LikelihoodBilbyInterface,
    WhittleLikelihood,
    compute_whittle_likelihood,
    log_likelihood,
    noise_weighted_inner_product,
)
