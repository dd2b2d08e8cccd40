"""NUMA placement report of host buffers (no GPU needed: the page query and
the sysfs reads are host-side)."""
import os

import pytest


@pytest.mark.skipif(not os.path.isdir("/sys/devices/system/node"), reason="no NUMA sysfs")
def test_numa_report_counts_sampled_pages():
    import torch
    from tucuda_gb300 import hostmem
    t = torch.ones(1 << 22, dtype=torch.uint8)   # 4 MiB, touched
    r = hostmem.numa_report({"buf": t})
    assert r["host_nodes"] and all(isinstance(n, int) for n in r["host_nodes"])
    hist = r["buffers"]["buf"]
    assert isinstance(hist, dict) and "error" not in hist
    assert sum(hist.values()) == 64
    assert all(k in {str(n) for n in r["host_nodes"]} for k in hist)
