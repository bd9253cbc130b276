"""Waveform producers (IMRPhenomD, IMRPhenomHM) feeding the response plugins,
and the post-Newtonian t(f) of the lalsimulation interface."""

from .interface_lalsim import get_PN_d_phase  # noqa: F401
from .phenomd import IMRPhenomD, PARAM_NAMES, theta_from_parameters  # noqa: F401
from .phenomhm import IMRPhenomHM  # noqa: F401
