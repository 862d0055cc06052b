"""The MATLAB / Octave gateway (voxhenry_gb300/mex/voxhenry_gpu_mex.c) built against a stub mex.h in
both complex layouts: it compiles warning-free, rejects bad calls with VoxHenryGPU:<status>
identifiers, and reports a missing device as an error (no fallback)."""
import os
import shutil
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "mex_stub"))
import gateway  # noqa: E402

pytestmark = pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc is needed to build the gateway")


@pytest.fixture(scope="module", params=[False, True], ids=["split", "interleaved"])
def gw(request, tmp_path_factory):
    import __graft_entry__

    __graft_entry__.build()
    g = gateway.Gateway(gateway.build(str(tmp_path_factory.mktemp("mex")), request.param))
    assert g.interleaved == request.param
    return g


def test_reset_needs_no_device(gw):
    gw("reset", nargout=0)


def test_bad_calls_raise_with_identifiers(gw):
    with pytest.raises(gateway.MexError) as e:
        gw(3.0)                                     # no command string
    assert e.value.identifier == "VoxHenryGPU:VH_ERR_BAD_ARG"


def test_no_device_is_an_error(gw):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(gateway.MexError) as e:
        gw("matvec", np.zeros(3), nargout=1)
    assert e.value.identifier == "VoxHenryGPU:VH_ERR_NO_DEVICE"
