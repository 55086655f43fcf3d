"""Serving-loop host logic on CPU: the device calls are replaced by fakes, so
what is checked is the scheduling, the latency bookkeeping and the summary."""
import pytest

from prothlogic_gb300 import serve


class _FakeBatch:
    """Finishes each submitted candidate after `n // 1000` calls of run()."""

    def __init__(self, max_slots):
        self.live = {}
        self.done = []
        self.budget = None

    def set_budget(self, b):
        self.budget = b

    def submit(self, k, n, tag):
        self.live[tag] = [k, n, max(1, n // 1000)]

    def pending(self):
        return 0, len(self.live), len(self.done)

    def run(self, steps):
        for tag in list(self.live):
            self.live[tag][2] -= 1
            if self.live[tag][2] == 0:
                k, n, _ = self.live.pop(tag)
                self.done.append({"tag": tag, "verdict": int(k == 3), "res64": k * n, "fft_len": 1024,
                                  "status": 0, "fft_bumps": 0})

    def poll(self):
        out, self.done = self.done, []
        return out

    def close(self):
        pass


class _FakePrefilter:
    """Answers a call on the second poll after it started (the work is 'running'
    for one loop turn); every candidate with k % 5 == 0 has the factor 5."""

    calls = []

    def __init__(self, bound=1 << 32, cap=65536):
        self.bound, self.cap = bound, cap
        self.cands = None
        self.turns = 0

    def busy(self):
        return self.cands is not None

    def start(self, cands):
        assert not self.busy() and len(cands) <= self.cap
        self.cands, self.turns = list(cands), 0
        _FakePrefilter.calls.append(len(cands))

    def poll(self):
        if not self.busy():
            return None
        self.turns += 1
        if self.turns < 2:
            return None
        out = [5 if k % 5 == 0 else 0 for k, _ in self.cands]
        self.cands = None
        return out

    def close(self):
        self.cands = None


def test_serve_bookkeeping(monkeypatch):
    _FakePrefilter.calls = []
    monkeypatch.setattr(serve, "Batch", _FakeBatch)
    monkeypatch.setattr(serve, "PrefilterStream", _FakePrefilter)
    arrivals = [(0.001 * i, 2 * i + 3, 2000 + 1000 * (i % 3)) for i in range(30)]
    recs, s = serve.serve(arrivals, budget_bytes=1 << 20, slice_steps=1, window=0.03)
    assert s["arrived"] == 30 and s["completed"] == 30
    rejected = [r for r in recs if not r["tested"]]
    assert {r["k"] for r in rejected} == {k for _, k, _ in arrivals if k % 5 == 0}
    assert all(r["factor"] == 5 for r in rejected)
    assert s["tested"] == 30 - len(rejected) and s["admitted"] == s["tested"] and s["unfinished"] == 0
    assert s["primes"] == sum(1 for r in recs if r["tested"] and r["k"] == 3)
    for r in recs:
        assert r["t_verdict"] >= r["t_arrive"]
    assert s["p99_s"] >= s["p50_s"] >= 0
    assert s["errors"] == 0
    assert sum(_FakePrefilter.calls) == 30  # every arrival went through the pre-filter once


def test_percentiles():
    assert serve._pct([], 50) is None
    xs = list(range(101))
    assert serve._pct(xs, 50) == 50 and serve._pct(xs, 99) == 99 and serve._pct(xs, 0) == 0


def test_time_limit_leaves_unfinished(monkeypatch):
    class _NoFactor(_FakePrefilter):
        def poll(self):
            out = super().poll()
            return None if out is None else [0] * len(out)

    monkeypatch.setattr(serve, "Batch", _FakeBatch)
    monkeypatch.setattr(serve, "PrefilterStream", _NoFactor)
    arrivals = [(0.0, 7, 10 ** 9)]  # would need a million slices
    recs, s = serve.serve(arrivals, time_limit=0.2, window=0.1)
    assert s["admitted"] == 1 and s["tested"] == 0 and s["unfinished"] == 1


def test_arrivals_during_a_prefilter_call_wait_for_the_next(monkeypatch):
    """Candidates arriving while a pre-filter call runs are held and sent together
    in the next call; the batch keeps running meanwhile."""
    _FakePrefilter.calls = []
    monkeypatch.setattr(serve, "Batch", _FakeBatch)
    monkeypatch.setattr(serve, "PrefilterStream", _FakePrefilter)
    arrivals = [(0.0, 7, 3000)] + [(0.0005 * i, 11 + 2 * i, 2000) for i in range(1, 20)]
    recs, s = serve.serve(arrivals, slice_steps=1, window=0.01)
    assert s["completed"] == 20
    assert sum(_FakePrefilter.calls) == 20 and max(_FakePrefilter.calls) <= 20
