"""ptxas's resource report of the library build (written beside each object by build.py): no
kernel spills registers to local memory, and the hot kernels are there with their launch-bound
register budgets.  Reads what the compiler prints (-Xptxas -v); no GPU needed."""
import glob
import os
import re

import pytest

BUILD = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "spatialops-threadfix_gb300",
                     "_build")
# hot kernel -> largest register count its occupancy plan allows
HOT = {
    "deep_out_kernel": 48,           # 5 blocks of 256 threads per SM
    "box_filter_kernel": 64,         # 4 blocks of 256
    "heat_step_f32x2_kernel": 80,    # 3 blocks of 256
    "heat_step_f32_bulk2_kernel": 80,  # 3 blocks of 256
    "transport_stage_f32_pair_kernel": 96,
    "patches_f32_strip_kernel": 128,  # 2 blocks of 256
}


def _report():
    files = sorted(glob.glob(os.path.join(BUILD, "*.o.resources.txt")))
    if not files:
        pytest.skip("library not built with resource reports")
    kernels = {}
    for f in files:
        name = None
        for ln in open(f):
            m = re.search(r"Compiling entry function '([^']+)'", ln)
            if m:
                name = m.group(1)
                kernels[name] = {}
                continue
            if name is None:
                continue
            m = re.search(r"(\d+) bytes spill stores, (\d+) bytes spill loads", ln)
            if m:
                kernels[name]["spill"] = int(m.group(1)) + int(m.group(2))
            m = re.search(r"Used (\d+) registers", ln)
            if m:
                kernels[name]["regs"] = int(m.group(1))
    return kernels


def test_no_kernel_spills():
    k = _report()
    spilled = {n: v["spill"] for n, v in k.items() if v.get("spill")}
    assert not spilled, spilled


@pytest.mark.parametrize("hot", sorted(HOT))
def test_hot_kernel_register_budget(hot):
    k = _report()
    found = {n: v for n, v in k.items() if hot in n}
    assert found, hot
    for n, v in found.items():
        assert v["regs"] <= HOT[hot], (n, v)
