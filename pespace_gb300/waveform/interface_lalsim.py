"""Post-Newtonian t(f) for lalsimulation waveforms (pespace/waveform/interface_lalsim.py).

The reference's lalsimulation interface fills the waveform container's
``tf`` entry for frequency-domain approximants with ``get_PN_d_phase``
(interface_lalsim.py:279-281, 297-482): t(f) = -(1/2 pi) dPsi/df of the
aligned-spin TaylorF2 phase, shifted so that t(f_ISCO) = 0 and zero above.
The same call here evaluates it on the GPU (``pes_pn_tf``, FP64); lalsuite
itself is not part of this package.
"""

import numpy as np
import torch

from .. import _lib

PN_PARAMS = ("mass_1", "mass_2", "spin_1z", "spin_2z")


def get_PN_d_phase(parameters, frequency_samples):
    """t(f) [s] at ``frequency_samples`` [Hz].

    parameters : mapping with mass_1, mass_2 (detector-frame solar masses),
        spin_1z, spin_2z; scalars give one system and an (n,) result, equal
        length 1-D arrays a batch and a (B, n) result.
    frequency_samples : (n,) frequencies (array or tensor).

    Returns a NumPy array (the reference's return type) for NumPy or list
    input, a CUDA tensor for tensor input.
    """
    values = [np.asarray(parameters[k].detach().cpu() if isinstance(parameters[k], torch.Tensor) else parameters[k],
                         dtype=np.float64) for k in PN_PARAMS]
    shape = np.broadcast_shapes(*(v.shape for v in values))
    if len(shape) > 1:
        raise ValueError(f"get_PN_d_phase: parameters must be scalars or 1-D arrays, got shape {shape}")
    single = shape == ()
    params = np.ascontiguousarray(np.stack([np.broadcast_to(v, shape).reshape(-1) for v in values], axis=1))
    tensor_in = isinstance(frequency_samples, torch.Tensor)
    freqs = torch.as_tensor(np.asarray(frequency_samples.detach().cpu() if tensor_in else frequency_samples,
                                       dtype=np.float64), device="cuda").reshape(-1).contiguous()
    B, n = params.shape[0], freqs.numel()
    d_params = torch.as_tensor(params, device="cuda")
    out = torch.empty((B, n), dtype=torch.float64, device="cuda")
    lib = _lib.load()
    for lo in range(0, B, 65535):
        b = min(65535, B - lo)
        _lib.check(lib.pes_pn_tf(_lib.ptr(d_params[lo:lo + b]), b, _lib.ptr(freqs), n, _lib.ptr(out[lo:lo + b]),
                                 _lib.stream_handle()))
    res = out[0] if single else out
    return res if tensor_in else res.cpu().numpy()
