"""Groups of 2D solves advanced by shared launches (kb_group_* in the C ABI).

Serving many small 2D solves one handle at a time leaves the GPU mostly idle:
every step of every solve is a chain of small kernels.  A Group advances all
of its member handles with one launch of each step kernel per step; each
member keeps its own device state, joins and leaves between chunks of steps,
and its result is bit-identical to stepping it alone with GROUP_SHAPE.
Members: 2D FP32-split KCU solves (BGK or Shakhov, one model per group)
without ghost-filled boundaries -- the served lid-driven cavities.
"""
import ctypes
import time

import numpy as np

from . import _native as N

# the launch shapes the group runs its members with (Handle.set_tuning keys)
GROUP_SHAPE = dict(march_tx=2, march_ry=8, march_bs=128, mom_ts=2)


def groupable(handle):
    """A handle of the form the group kernels cover (the C ABI also refuses,
    with KB_ERR_CONFIG, grids too large for the group's 32-thread cell blocks)."""
    c = handle.cfg
    bc_ok = all(c.bc[k] in (N.BOUNDARY["fix"], N.BOUNDARY["maxwell"]) for k in range(4))
    return c.dim == 2 and c.precision == N.PRECISION["fp32"] and c.flux == N.FLUX["kcu"] and bc_ok


class Group:
    """A group of resident 2D solves stepped together."""

    def __init__(self, capacity=64):
        self.lib = N.load()
        g = ctypes.c_void_p()
        N.check(self.lib.kb_group_create(int(capacity), ctypes.byref(g)))
        self.g = g
        self.members = []  # Handle objects, member order of kb_group_query

    def close(self):
        if getattr(self, "g", None):
            self.lib.kb_group_destroy(self.g)
            self.g = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add(self, handle, dt):
        N.check(self.lib.kb_group_add(self.g, handle.h, float(dt)))
        self.members.append(handle)

    def remove(self, handle):
        N.check(self.lib.kb_group_remove(self.g, handle.h))
        self.members.remove(handle)

    def step_async(self, nsteps):
        N.check(self.lib.kb_group_step_async(self.g, int(nsteps)))

    def query(self):
        """(ready, residual [members][4], status [members]) of the last chunk."""
        n = len(self.members)
        res = np.zeros((max(n, 1), 4))
        st = np.zeros(max(n, 1), dtype=np.int32)
        ready = ctypes.c_int32()
        N.check(self.lib.kb_group_query(self.g, N.ptr(res), st.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                        ctypes.byref(ready)))
        return bool(ready.value), res[:n], st[:n]

    def wait(self, timeout=None):
        """Poll until the last chunk is done; TimeoutError after `timeout`
        seconds (None: no limit)."""
        t_end = None if timeout is None else time.monotonic() + timeout
        while True:
            ready, res, st = self.query()
            if ready:
                return res, st
            if t_end is not None and time.monotonic() > t_end:
                raise TimeoutError("group chunk not done after %.3g s" % timeout)
            time.sleep(0)

    def launches(self):
        n, l = ctypes.c_int32(), ctypes.c_int64()
        N.check(self.lib.kb_group_info(self.g, ctypes.byref(n), ctypes.byref(l)))
        return l.value
