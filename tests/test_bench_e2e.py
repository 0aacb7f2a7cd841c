"""bench.py's end-to-end measurement on CPU with a stand-in context: three
timed windows per call kind, each ending on a rebuild step, the median
reported, and the host path of every timed call counted as the library
reports it."""
import ctypes
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


class FakeCtx:
    """The calls measure_e2e makes, with the host path a GB300 context reports
    (kernels' direct access on rebuild steps, copy-engine chunks otherwise)."""

    def __init__(self):
        self.step = -1
        self.closed = False

    def forward_host_batch(self, W, pos, boxes, step, flags, s, d, v):
        self.step = step
        for w in range(W):
            ctypes.c_double.from_address(s + 8 * w).value = 1.0
        time.sleep(1e-4)

    def forward_host(self, pos, box, step, flags, s, d, v):
        self.step = step
        ctypes.c_double.from_address(s).value = 1.0
        time.sleep(1e-5)

    def nl_size(self, frame=0):
        return 1000 + 10 * (self.step // 10)

    def host_path(self):
        return "direct" if self.step % 10 == 0 else "chunked"

    def close(self):
        self.closed = True


def test_measure_e2e_windows_and_paths():
    import bench
    from plumed2_gb300._lib import addr
    W, n, T = 3, 8, 10
    hp = np.random.default_rng(0).normal(size=(T, W, n, 3))
    hs, hd, hv = np.zeros(W), np.zeros((W, n, 3)), np.zeros((W, 9))
    made = []

    def make():
        made.append(FakeCtx())
        return made[-1]

    v, wins, bpaths, vw, wwins, wpaths = bench.measure_e2e(make, hp, hs, hd, hv, np.eye(3) * 2.0, W, n, 10, addr)
    assert len(wins) == bench.E2E_WINDOWS == 3 and len(wwins) == 3
    assert v == float(np.median(wins)) and vw == float(np.median(wwins))
    assert all(x > 0 for x in wins + wwins)
    # 30 timed batched calls: the rebuilds at steps 20, 30, 40 went direct
    assert bpaths == {"chunked": 27, "direct": 3}
    assert wpaths == {"chunked": 27 * W, "direct": 3 * W}
    assert len(made) == 1 + W and all(c.closed for c in made)
    note = bench.host_path_note(bpaths)
    assert note.startswith(bench.HOST_PATH_TEXT["chunked"] + ": 27 of 30 calls")
    assert bench.HOST_PATH_TEXT["direct"] + ": 3 of 30 calls" in note


def test_e2e_pairs_counts_the_rebuilt_lists():
    import bench
    # ten steps after a build: nine on the old lists, the rebuild step on the new
    assert bench.e2e_pairs(100, 120, 10) == 9 * 100 + 120
