"""The open-loop serving driver (voxel-rt_gb300/serving.py) against a fake server on the
CPU: requests go in by arrival time and in order, the driver waits on the server between
arrivals instead of sleeping past completions, and the summary's percentiles and rates
come from the completions it gets back."""
import numpy as np

import serving
import vrt


class FakeServer:
    """Completes every submitted request after `latency_ms` of the driver's clock."""

    def __init__(self, latency_ms: float = 0.3):
        self.latency_ms = latency_ms
        self.submitted = []   # (tag, kind, world_id, submit time)
        self.pending = []
        self.waits = 0
        self.t0 = None

    def _now(self):
        import time
        if self.t0 is None:
            self.t0 = time.perf_counter()
        return (time.perf_counter() - self.t0) * 1e3

    def submit(self, q):
        t = self._now()
        self.submitted.append((int(q.user_tag), int(q.kind), int(q.world_id), t))
        self.pending.append((q.user_tag, q.kind, t))

    def poll(self):
        now = self._now()
        out, keep = [], []
        for tag, kind, t in self.pending:
            if now - t >= self.latency_ms:
                c = vrt.Completion()
                c.user_tag, c.kind, c.status = tag, kind, 0
                c.submit_ms, c.start_ms, c.done_ms = t, t, now
                c.rays = 1000 if kind == vrt.REQ_RENDER else 0
                out.append(c)
            else:
                keep.append((tag, kind, t))
        self.pending = keep
        return out

    def wait(self, timeout_us):
        import time
        self.waits += 1
        if not self.pending:
            return False
        end = time.perf_counter() + timeout_us * 1e-6
        while time.perf_counter() < end:
            if any(self._now() - t >= self.latency_ms for _, _, t in self.pending):
                return True
        return False

    def drain(self):
        import time
        out = []
        while self.pending:
            time.sleep(0.0001)
            out += self.poll()
        return out


def make_stream(n=60, gap_s=0.002):
    u = vrt.default_uniforms()
    reqs = []
    for i in range(n):
        if i % 10 == 9:
            reqs.append((i * gap_s, vrt.REQ_EDIT, i % 2, (5, 6, 7, 3)))
        else:
            reqs.append((i * gap_s, vrt.REQ_RENDER, i % 2, (u, 64, 48)))
    return reqs


def test_requests_go_in_order_and_complete():
    srv = FakeServer()
    reqs = make_stream()
    done, wall = serving.run_open_loop(srv, [10, 11], reqs)
    tags = [s[0] for s in srv.submitted]
    assert tags == list(range(len(reqs)))                      # arrival order
    assert [s[2] for s in srv.submitted] == [10 + (i % 2) for i in range(len(reqs))]
    assert all(s[3] + 1.0 >= 1e3 * reqs[s[0]][0] for s in srv.submitted)  # never before arrival (1 ms slack)
    assert sorted(int(c.user_tag) for c in done) == list(range(len(reqs)))
    assert srv.waits > 0                                        # the driver waited on the server
    assert wall >= reqs[-1][0]


def test_summary_counts_and_percentiles():
    done = []
    for i, lat in enumerate([0.1, 0.2, 0.3, 0.4, 10.0]):
        c = vrt.Completion()
        c.user_tag, c.kind, c.status, c.submit_ms, c.done_ms, c.rays = i, vrt.REQ_RENDER, 0, 5.0, 5.0 + lat, 2_000_000
        done.append(c)
    e = vrt.Completion()
    e.kind, e.status = vrt.REQ_EDIT, 0
    refused = vrt.Completion()
    refused.kind, refused.status = vrt.REQ_RENDER, vrt.EBUDGET
    s = serving.summarize(done + [e, refused], wall_s=0.5)
    assert s["renders"] == 5 and s["edits"] == 1 and s["refused"] == 1
    assert np.isclose(s["p50_ms"], 0.3) and s["p99_ms"] > 9.0
    assert np.isclose(s["mrays_per_s"], 5 * 2_000_000 / 0.5 / 1e6)
    assert serving.summarize([], 1.0) == {"renders": 0}
