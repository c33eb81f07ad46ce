"""pn_measure_pipe_rates: every rate is measured (positive, finite) and the
FP32 FMA rate stays under the part's issue limit (four warp instructions per
SM per clock at 2.1 GHz at most), so each figure is a plausible rate of the
kernel that claims it rather than a loop the compiler removed."""
import math

import pytest

from pannde_gb300.solver import PIPE_RATE_NAMES, measure_pipe_rates

pytestmark = pytest.mark.gpu


def test_pipe_rates(cuda_device):
    import torch
    r = measure_pipe_rates()
    assert set(r) == set(PIPE_RATE_NAMES)
    sms = torch.cuda.get_device_properties(0).multi_processor_count
    ceiling = sms * 4 * 32 * 2.2e9  # thread-operations per second at full issue
    for k, v in r.items():
        assert math.isfinite(v) and 0 < v <= ceiling, (k, v)
    # the FP32 FMA pipe is at least as fast as the FP64 one on every part
    assert r["fp32_fma"] >= r["fp64_fma"]
    print({k: f"{v:.3e}" for k, v in r.items()})
