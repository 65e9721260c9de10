"""Bounded waits: a wait that runs out returns an error status, the context lives on.

Every spin in the library's kernels (the F-engine's TMA mbarrier waits, the
tensor-core engine's MMA/TMEM waits) goes through a clock-bounded wait that
records a watchdog code and returns. Here the self-test kernel waits on an
mbarrier nothing completes, with a short budget; the host must see
CORR_ERR_INTERNAL from corrx_check, and the engine must keep working after.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_watchdog_timeout_is_reported_and_recoverable(pkg, cuda, oracle):
    torch = cuda
    eng = pkg.FxEngine(2, 1024, max_frames=4)
    h = eng.lib
    assert h.corrx_selftest_watchdog(eng.h, 200000, None) == 0   # ~0.1 ms budget
    with pytest.raises(pkg.CorrError) as e:
        eng.check()
    assert e.value.status == pkg.abi.CORR_ERR_INTERNAL
    assert "watchdog" in e.value.message
    eng.check()   # the flag was cleared; nothing is pending
    # and the engine still computes correctly
    x = np.random.default_rng(0).integers(-20, 20, size=(2, 3, 2048)).astype(np.int8)
    acc = eng.new_acc()
    eng.accumulate(torch.from_numpy(x).cuda(), 3, acc)
    torch.cuda.synchronize()
    eng.check()
    assert oracle.rel_rms(acc.cpu().numpy(), oracle.correlate(x)) < 1e-5
    eng.close()
