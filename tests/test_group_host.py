"""kitgpu.group.Group's host side on the CPU with a fake library in place of
libkitgpu's kb_group_* calls: member bookkeeping, query results trimmed to
the members, launch counts, and a wait that gives up after its timeout
instead of polling forever when a chunk never completes."""
import ctypes

import numpy as np
import pytest

from kitgpu import _native as N
from kitgpu import group as G


class FakeLib:
    def __init__(self, done_after):
        self.members = []
        self.polls = 0
        self.done_after = done_after  # polls until the chunk is done (None: never)
        self.launched = 0

    def kb_group_create(self, cap, out):
        out._obj.value = 1
        return 0

    def kb_group_destroy(self, g):
        return 0

    def kb_group_add(self, g, h, dt):
        self.members.append(h)
        return 0

    def kb_group_remove(self, g, h):
        self.members.remove(h)
        return 0

    def kb_group_step_async(self, g, n):
        self.polls = 0
        self.launched += 8 * n
        return 0

    def kb_group_query(self, g, res, st, ready):
        self.polls += 1
        done = self.done_after is not None and self.polls > self.done_after
        ready._obj.value = int(done)
        if done:
            r = np.ctypeslib.as_array(res, shape=(max(len(self.members), 1), 4))
            for k in range(len(self.members)):
                r[k] = k + 1
        return 0

    def kb_group_info(self, g, n, l):
        n._obj.value = len(self.members)
        l._obj.value = self.launched
        return 0


class H:
    def __init__(self, k):
        self.h = ctypes.c_void_p(100 + k)


@pytest.fixture
def fake(monkeypatch):
    def install(done_after):
        lib = FakeLib(done_after)
        monkeypatch.setattr(N, "load", lambda: lib)
        return lib
    return install


def test_members_query_and_launches(fake):
    lib = fake(done_after=3)
    g = G.Group(capacity=4)
    a, b, c = H(0), H(1), H(2)
    for h in (a, b, c):
        g.add(h, 1e-3)
    g.remove(b)
    assert g.members == [a, c]
    g.step_async(5)
    res, st = g.wait(timeout=5.0)
    assert res.shape == (2, 4) and np.array_equal(res[:, 0], [1, 2]) and st.shape == (2,)
    assert g.launches() == 40
    g.close()


def test_wait_gives_up_after_its_timeout(fake):
    fake(done_after=None)
    g = G.Group()
    g.add(H(0), 1e-3)
    g.step_async(1)
    with pytest.raises(TimeoutError):
        g.wait(timeout=0.05)
    ready, _, _ = g.query()
    assert not ready
    g.close()
