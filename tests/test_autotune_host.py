"""Launch options and the autotuner: host-side checks (no plan, no GPU)."""

import ctypes
import types

import pytest


def test_option_entry_points_reject_null_plan():
    from pespace_gb300 import _lib

    lib = _lib.load()
    v = ctypes.c_int64()
    assert lib.pes_plan_set_option(None, _lib.PES_OPT_DENSE_STAGE, 1) == _lib.PES_EINVAL
    assert b"null plan" in lib.pes_last_error()
    assert lib.pes_plan_get_option(None, _lib.PES_OPT_SAMPLE_THREADS, ctypes.byref(v)) == _lib.PES_EINVAL
    assert lib.pes_plan_get_option(None, 99, ctypes.byref(v)) == _lib.PES_EINVAL


def test_autotune_argument_checks():
    from pespace_gb300.inference.autotune import CANDIDATES, OPTIONS, autotune

    assert set(CANDIDATES) == set(OPTIONS)
    fake = types.SimpleNamespace(precision="mixed", max_batch=4)
    with pytest.raises(ValueError):
        autotune(fake, None, reps=0)
    with pytest.raises(ValueError):
        autotune(fake, None, candidates={"tile": (1, 2)})


def test_reference_constructor_rejects_other_waveforms():
    from pespace_gb300.inference import WhittleLikelihoodCuda

    with pytest.raises(TypeError):
        WhittleLikelihoodCuda("IMRPhenomXAS", None, ("A", "E", "T"))


def test_option_codes_match_header():
    import os
    import re

    from pespace_gb300 import _lib

    with open(os.path.join(os.path.dirname(__file__), "..", "include", "pespace_gb300.h")) as fh:
        codes = dict(re.findall(r"#define (PES_OPT_\w+) (\d+)", fh.read()))
    assert set(codes) == {"PES_OPT_DENSE_STAGE", "PES_OPT_SAMPLE_THREADS", "PES_OPT_REFINE_ALL"}
    assert all(getattr(_lib, k) == int(v) for k, v in codes.items())
