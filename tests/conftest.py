"""Shared test helpers.  `gpu`-marked tests run on a GB300; everything else runs on a CPU."""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (run on the GB300)")


def rel_err(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def make_case(dims, Ls, nsimd=1, gseeds=(1, 2, 3, 4), fseeds=(5, 6, 7, 8)):
    import gridbench_gb300 as gb
    U = gb.generate_gauge(dims, nsimd, gseeds)
    phi = gb.generate_fermion(dims, Ls, nsimd, fseeds)
    nbr, prm, nsite = gb.generate_table(dims, Ls, nsimd)
    return {"dims": tuple(dims), "Ls": Ls, "nsimd": nsimd, "U": U, "phi": phi, "nbr": nbr, "prm": prm,
            "nsite": nsite}


@pytest.fixture(scope="session")
def gpu():
    """The CUDA library, failing loudly when no device is visible."""
    import gridbench_gb300 as gb
    gb.load()
    if not gb.device_available():
        pytest.fail("gpu-marked test but no CUDA device is visible: " + gb.load().gbdw_last_error().decode())
    return gb


def host_memory_available() -> float:
    """Bytes this process may still allocate on the host: MemAvailable, capped by the cgroup
    limit when one is set (the big-lattice parity tests check it before they start)."""
    avail = float("inf")
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                avail = float(line.split()[1]) * 1024
    except OSError:
        pass
    for lim, cur in (("/sys/fs/cgroup/memory.max", "/sys/fs/cgroup/memory.current"),
                     ("/sys/fs/cgroup/memory/memory.limit_in_bytes", "/sys/fs/cgroup/memory/memory.usage_in_bytes")):
        try:
            raw = open(lim).read().strip()
            if raw != "max" and float(raw) < 1e18:
                avail = min(avail, float(raw) - float(open(cur).read().strip()))
            break
        except (OSError, ValueError):
            continue
    return avail


def need_host_memory(nbytes: float):
    have = host_memory_available()
    if have < nbytes:
        pytest.skip(f"needs {nbytes / 2**30:.1f} GiB of host memory, {have / 2**30:.1f} GiB available")
