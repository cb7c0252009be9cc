"""Measured tensor-path rates of the GPU the tests run on: FP64 (DMMA,
DFMA) and the warp-level INT8 and bf16 mma.sync paths.  The numbers are
printed for the record; the test checks only that each measurement ran and
is positive (no rate is assumed)."""
import pytest

pytestmark = pytest.mark.gpu


def test_rates_measured(world):
    dmma, dfma = world.fp64_rates()
    imma, hmma = world.mma_sync_rates()
    print(f"DMMA {dmma:.2f} TFLOP/s, DFMA {dfma:.2f} TFLOP/s, "
          f"INT8 mma.sync {imma:.1f} TOP/s, bf16 mma.sync {hmma:.1f} TFLOP/s")
    assert dmma > 0 and dfma > 0 and imma > 0 and hmma > 0
