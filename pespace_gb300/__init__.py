"""pespace_gb300: GB300 (sm_103a) CUDA implementation of pespace's frequency-domain
response, TDI and Whittle-likelihood path behind a C ABI (include/pespace_gb300.h).

Subpackages mirror the reference layout: ``detector`` (orbit, noise, tdi,
antenna), ``waveform`` (IMRPhenomD producer) and ``inference`` (likelihoods).
"""

from . import build  # noqa: F401
from ._lib import PesError, library_path, load  # noqa: F401

__version__ = "0.1.0"
