"""Waveform producers (IMRPhenomD) feeding the response plugins."""

from .phenomd import IMRPhenomD, PARAM_NAMES, theta_from_parameters  # noqa: F401
