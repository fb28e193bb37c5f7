"""No C++ exception leaves a C entry point: a host allocation that fails
inside the library comes back as PT_ERR_OOM with a message, and the process
goes on (where an escaping std::bad_alloc would abort it).  The failure is
made on the host: a child process caps its own address space just above what
it uses and asks the world builder for a 256 MB atlas layer copy."""
import subprocess
import sys
import textwrap
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

CHILD = textwrap.dedent("""
    import ctypes as C, resource, sys
    sys.path[:0] = [{root!r}, {pkg!r}]
    import numpy as np
    import pathtracer as pt
    from pathtracer import abi
    lib = pt.load()
    layer = np.zeros(abi.PT_ATLAS_SIZE * abi.PT_ATLAS_SIZE * 4, np.uint8)  # the caller's texels, allocated first
    w = C.c_void_p()
    assert lib.ptw_create(C.byref(w)) == abi.PT_OK
    size = int(open("/proc/self/statm").read().split()[0]) * resource.getpagesize()
    resource.setrlimit(resource.RLIMIT_AS, (size + (64 << 20), resource.RLIM_INFINITY))
    index = C.c_int32()
    rc = lib.ptw_add_atlas_layer(w, 1, layer.ctypes.data, C.byref(index))
    resource.setrlimit(resource.RLIMIT_AS, (resource.RLIM_INFINITY, resource.RLIM_INFINITY))
    print(rc, lib.ptw_last_error(w).decode(errors="replace"))
    lib.ptw_destroy(w)
""")


@pytest.mark.skipif(not sys.platform.startswith("linux"), reason="address-space limit through /proc and rlimit")
def test_failed_host_allocation_is_a_status_not_an_abort():
    from pathtracer import abi
    code = CHILD.format(root=str(ROOT), pkg=str(ROOT / "path-tracer_gb300"))
    proc = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr[-2000:]
    rc, _, message = proc.stdout.strip().splitlines()[-1].partition(" ")
    assert int(rc) == abi.PT_ERR_OOM and "out of host memory" in message
