"""NUMA placement of page-locked host buffers relative to the GPU.

The host-image paths copy from and to pinned host slabs; the rate of those
copies depends on the slabs sitting on the NUMA node the GPU is attached to.
``numa_report`` reads the GPU's node from sysfs and asks the kernel
(``move_pages`` with no target nodes, a query) which node holds a sample of
each buffer's pages.  Linux only; other systems get ``{"available": False}``.
"""
import ctypes
import os
import subprocess

_SYS_MOVE_PAGES = {"aarch64": 239, "x86_64": 279}


def _pages_nodes(ptr, nbytes, samples=64):
    """Histogram {node: pages} of `samples` pages spread over [ptr, ptr+nbytes)."""
    nr = _SYS_MOVE_PAGES.get(os.uname().machine)
    if nr is None or nbytes <= 0:
        return None
    page = os.sysconf("SC_PAGE_SIZE")
    step = max(page, (nbytes // samples) // page * page)
    base = ptr // page * page
    addrs = [base + i * step for i in range(samples) if i * step < nbytes]
    pages = (ctypes.c_void_p * len(addrs))(*addrs)
    status = (ctypes.c_int * len(addrs))()
    libc = ctypes.CDLL(None, use_errno=True)
    if libc.syscall(nr, 0, ctypes.c_ulong(len(addrs)), pages, None, status, 0) != 0:
        return {"error": os.strerror(ctypes.get_errno())}
    hist = {}
    for s in status:
        key = str(s) if s >= 0 else f"err{-s}"
        hist[key] = hist.get(key, 0) + 1
    return hist


def gpu_numa_node(device_index=0):
    """NUMA node of the GPU's PCI device (-1: none reported), or None."""
    try:
        bus = subprocess.run(["nvidia-smi", "--query-gpu=pci.bus_id", "--format=csv,noheader",
                              "-i", str(device_index)], capture_output=True, text=True,
                             timeout=30).stdout.strip()
        dom, rest = bus.split(":", 1)
        with open(f"/sys/bus/pci/devices/{(dom[-4:] + ':' + rest).lower()}/numa_node") as f:
            return int(f.read().strip())
    except (OSError, ValueError, subprocess.SubprocessError):
        return None


def numa_report(buffers, device_index=0):
    """{"gpu_node", "host_nodes", "buffers": {name: {node: pages}}} for a dict
    of named CPU tensors (pinned slabs)."""
    if not os.path.isdir("/sys/devices/system/node"):
        return {"available": False}
    nodes = sorted(int(d[4:]) for d in os.listdir("/sys/devices/system/node")
                   if d.startswith("node") and d[4:].isdigit())
    return {"gpu_node": gpu_numa_node(device_index), "host_nodes": nodes,
            "buffers": {name: _pages_nodes(t.data_ptr(), t.numel() * t.element_size())
                        for name, t in buffers.items()}}
