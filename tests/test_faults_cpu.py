"""Host-side fault injection without a GPU: MDRL_FAULT makes a named CUDA runtime call of
mdrl_create report failure before the call is made, so the error path is exercised on a machine
with no GPU (the GPU-side tests cover every other entry point)."""
import os

import pytest

import sc2019_md_gb300 as m


@pytest.fixture
def fault_env():
    old = os.environ.get("MDRL_FAULT")
    yield
    if old is None:
        os.environ.pop("MDRL_FAULT", None)
    else:
        os.environ["MDRL_FAULT"] = old


def test_create_reports_the_injected_call(fault_env):
    os.environ["MDRL_FAULT"] = "create:cudaGetDeviceCount"
    with pytest.raises(m.MdrlError) as e:
        m.Context(m.default_params())
    assert e.value.status == 4
    assert "cudaGetDeviceCount" in str(e.value) and "injected" in str(e.value)


def test_count_and_scope_of_the_switch(fault_env):
    """'@k' fails the k-th matching call only, and a spec without 'create:' is not armed inside
    mdrl_create: neither reports an injected failure (without a GPU the real call then fails)."""
    for spec in ("create:cudaGetDeviceCount@2", "cudaGetDeviceCount", ""):
        os.environ["MDRL_FAULT"] = spec
        try:
            m.Context(m.default_params()).close()
        except m.MdrlError as e:
            assert "injected" not in str(e), spec


def test_validation_precedes_any_cuda_call(fault_env):
    """Invalid parameters are rejected before the first CUDA call, armed fault or not."""
    os.environ["MDRL_FAULT"] = "create:cudaGetDeviceCount"
    p = m.default_params()
    p.cutoff = -1.0
    with pytest.raises(m.MdrlError) as e:
        m.Context(p)
    assert e.value.status == 1
    p = m.default_params()
    p.coulomb_k = float("inf")
    with pytest.raises(m.MdrlError) as e:
        m.Context(p)
    assert e.value.status == 1 and "coulomb_k" in str(e.value)
