"""The reference's public names on the path, including its placeholders:
plugin interfaces, placeholder models that are not implemented there either,
unimplemented data-container conversions, the taichi-suffixed likelihood
name (CPU, no device)."""

import pytest


def test_plugin_interfaces():
    from pespace_gb300.detector.antenna import FDResponseModelMarset2018, SingleLinkResponseModel
    from pespace_gb300.detector.tdi import (FDMichelsonConstantEqualArm, TDICombinationModel,
                                            TDMichelsonConstantEqualArm)

    assert isinstance(FDResponseModelMarset2018(), SingleLinkResponseModel)
    assert isinstance(FDMichelsonConstantEqualArm(), TDICombinationModel)
    assert isinstance(TDMichelsonConstantEqualArm(), TDICombinationModel)
    with pytest.raises(TypeError):
        SingleLinkResponseModel()
    with pytest.raises(TypeError):
        TDICombinationModel()


@pytest.mark.parametrize("name", ["FDResponseModelLongWavelength", "FDResponseModelStaticLongWavelength"])
def test_placeholder_response_models(name):
    from pespace_gb300.detector import antenna

    with pytest.raises(TypeError):  # abstract, as the reference's placeholder
        getattr(antenna, name)()


def test_placeholder_tdi_model_and_container_stubs():
    from pespace_gb300.detector.tdi import FDMichelsonConstantEqualArmFFT, TDIChannelData

    with pytest.raises(TypeError):
        FDMichelsonConstantEqualArmFFT()
    td = TDIChannelData()
    for name in ("add_into_td_data", "add_into_wd_data"):
        with pytest.raises(NotImplementedError):
            getattr(td, name)()
    assert td.wd_data_numpy is None


def test_taichi_named_likelihood_call():
    from pespace_gb300.inference import compute_whittle_likelihood, compute_whittle_likelihood_ti

    assert compute_whittle_likelihood_ti is compute_whittle_likelihood
