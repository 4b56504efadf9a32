"""Device selection (src/correlation.cpp:163-175 setDevice/getDevice) and the
load-time entry points kept for R/zzz.R."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_set_and_get_device(gpu):
    import gputools_gb300 as g
    assert g.chooseGpu(0) == 0
    assert g.getGpuId() == 0


def test_invalid_device_reports_reference_message(gpu):
    bad = ctypes.c_int(999)
    gpu.rsetDevice(ctypes.byref(bad))
    assert "The gpu id number is not valid." in gpu.gt_last_error().decode()
    d = ctypes.c_int(-1)
    gpu.rgetDevice(ctypes.byref(d))
    assert d.value == 0


def test_cucompile_and_unload_are_harmless(gpu):
    n = ctypes.c_int(0)
    gpu.cuCompile(ctypes.byref(n), None, None)
    assert gpu.gt_last_error().decode() == ""
    gpu.unloadPackage()
    gpu.gt_release_workspace()
