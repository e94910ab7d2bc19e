"""Scheduling logic of the serving loop on a simulated device (CPU only).

The simulated backend gives each request a duration proportional to its
walkers x electrons and completes it when a manual clock passes that time, so
admission, slot assignment, the HBM budget and per-job ordering are checked
without a GPU.
"""
import numpy as np
import pytest

from jaqmc_gb300 import serving as SV
from jaqmc_gb300 import systems as S


class Clock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeBackend:
    def __init__(self, clock, footprint=lambda sp: 1000, req_bytes=lambda sp: 100 * sp.mol.n_electrons):
        self.clock = clock
        self.footprint = footprint
        self.req_bytes = req_bytes
        self.inflight = {}
        self.log = []
        self.captures = 0
        self.replays = 0
        self.allocated = 0

    def new_stream(self):
        return object()

    def job_footprint(self, spec):
        return self.footprint(spec)

    def request_bytes(self, spec):
        return self.req_bytes(spec)

    def create_job(self, spec):
        return {"spec": spec, "count": 0}

    def release_job(self, h):
        h["released"] = True

    def new_workspace(self, nbytes, stream):
        self.allocated += nbytes
        return ("ws", nbytes)

    def free_workspace(self, ws):
        if ws is not None:
            self.allocated -= ws[1]

    def _run(self, h, stream):
        sp = h["spec"]
        end = self.clock() + 1e-6 * sp.walkers * sp.mol.n_electrons
        self.inflight[id(stream)] = end
        h["count"] += 1
        self.log.append((self.clock(), sp.job_id, h["count"]))

    def run_request(self, h, ws, ws_bytes, stream):
        assert ws_bytes >= self.req_bytes(h["spec"])
        self._run(h, stream)
        self._last = h

    def capture(self, h, ws, ws_bytes, stream):
        self.captures += 1
        return (h, stream)

    def replay(self, g, stream):
        self.replays += 1
        self._run(g[0], stream)

    def record(self, stream):
        return self.inflight[id(stream)]

    def query(self, ev):
        return self.clock() >= ev

    def result(self, h):
        return np.array([h["spec"].job_id, h["count"], 0.0])


def _serve(server, clock, specs, dt=1e-4, limit=100000):
    specs = sorted(specs, key=lambda s: s.arrival)
    i = 0
    for _ in range(limit):
        while i < len(specs) and specs[i].arrival <= clock():
            server.arrive(specs[i])
            i += 1
        server.step()
        inflight = [s.request for s in server.slots if s.request is not None]
        assert len({r.job_id for r in inflight}) == len(inflight)
        assert server.used <= server.budget
        if i == len(specs) and not server.busy():
            return
        clock.t += dt
    raise AssertionError("did not finish")


def test_all_requests_complete_in_order():
    clock = Clock()
    be = FakeBackend(clock)
    srv = SV.Server(be, n_slots=3, hbm_budget=1 << 30, clock=clock)
    specs = SV.atom_job_specs(12, rate=2000.0, seed=3, requests=4)
    _serve(srv, clock, specs)
    assert len(srv.finished_jobs) == 12
    for st in srv.finished_jobs:
        counts = [int(r[1]) for r in st.results]
        assert counts == [1, 2, 3, 4]
    assert len(srv.finished) == 48
    lat = srv.request_latencies_ms()
    assert np.all(lat > 0)
    # graphs: first request of each (job, slot) pair eager, the others replayed
    assert be.captures + be.replays == 48
    assert be.replays > 0


def test_overlap_uses_all_slots():
    clock = Clock()
    be = FakeBackend(clock)
    srv = SV.Server(be, n_slots=4, hbm_budget=1 << 30, clock=clock)
    specs = [SV.JobSpec(j, S.atom(6), 1024, requests=2, seed=j) for j in range(8)]
    peak = 0
    for sp in specs:
        srv.arrive(sp)
    while srv.busy():
        srv.step()
        peak = max(peak, sum(s.request is not None for s in srv.slots))
        clock.t += 1e-4
    assert peak == 4


def test_admission_waits_for_budget():
    clock = Clock()
    be = FakeBackend(clock, footprint=lambda sp: 600, req_bytes=lambda sp: 300)
    srv = SV.Server(be, n_slots=4, hbm_budget=1000, clock=clock)
    specs = [SV.JobSpec(j, S.atom(4), 512, requests=2, seed=j) for j in range(3)]
    _serve(srv, clock, specs)
    # only one 600-byte job fits next to a 300-byte workspace
    admitted = sorted(st.admitted for st in srv.finished_jobs)
    finished = sorted(st.finished for st in srv.finished_jobs)
    assert admitted[1] >= finished[0] and admitted[2] >= finished[1]
    assert srv.peak_used <= 1000


def test_job_larger_than_budget_is_rejected():
    clock = Clock()
    be = FakeBackend(clock, footprint=lambda sp: 2000)
    srv = SV.Server(be, n_slots=2, hbm_budget=1000, clock=clock)
    srv.arrive(SV.JobSpec(0, S.atom(3), 256))
    with pytest.raises(MemoryError):
        srv.step()


def test_slot_prefers_same_electron_count():
    clock = Clock()
    be = FakeBackend(clock)
    srv = SV.Server(be, n_slots=1, hbm_budget=1 << 30, clock=clock, use_graphs=False)
    specs = [SV.JobSpec(0, S.atom(6), 256, requests=1, seed=0),
             SV.JobSpec(1, S.atom(10), 256, requests=1, seed=1),
             SV.JobSpec(2, S.atom(6), 256, requests=1, seed=2)]
    for sp in specs:
        srv.arrive(sp)
    _serve(srv, clock, [])
    order = [j for _, j, _ in be.log]
    assert order == [0, 2, 1]


def test_workspace_shrinks_for_starved_request():
    clock = Clock()
    be = FakeBackend(clock, footprint=lambda sp: 10, req_bytes=lambda sp: 100 * sp.mol.n_electrons)
    srv = SV.Server(be, n_slots=2, hbm_budget=2000, clock=clock)
    # two small jobs leave 2 slots with 200-byte workspaces; a job needing 1800 must still run
    specs = [SV.JobSpec(0, S.atom(2), 256, requests=1), SV.JobSpec(1, S.atom(2), 256, requests=1),
             SV.JobSpec(2, S.atom(18), 256, requests=1, arrival=0.01)]
    _serve(srv, clock, specs)
    assert len(srv.finished_jobs) == 3


class PackingBackend(FakeBackend):
    """FakeBackend that also runs packed groups (one launch set for requests
    of jobs sharing a model)."""

    def __init__(self, clock, **kw):
        super().__init__(clock, **kw)
        self.groups = []

    def model_key(self, spec):
        return (spec.mol.n_electrons, spec.params_seed)

    def group_request_bytes(self, specs):
        return sum(self.req_bytes(sp) for sp in specs)

    def run_group(self, hs, ws, ws_bytes, stream):
        assert ws_bytes >= self.group_request_bytes([h["spec"] for h in hs])
        assert len({self.model_key(h["spec"]) for h in hs}) == 1
        self.groups.append([h["spec"].job_id for h in hs])
        end = self.clock() + 1e-6 * sum(h["spec"].walkers for h in hs) * hs[0]["spec"].mol.n_electrons
        self.inflight[id(stream)] = end
        for h in hs:
            h["count"] += 1
            self.log.append((self.clock(), h["spec"].job_id, h["count"]))


def test_requests_of_a_shared_model_are_packed():
    clock = Clock()
    be = PackingBackend(clock)
    srv = SV.Server(be, n_slots=1, hbm_budget=1 << 30, clock=clock, group_max=4)
    # six jobs of one model (carbon, parameters seed 0), two of another
    specs = [SV.JobSpec(j, S.atom(6), 256, requests=2, seed=j, param_seed=0) for j in range(6)]
    specs += [SV.JobSpec(6 + j, S.atom(8), 256, requests=2, seed=6 + j, param_seed=0) for j in range(2)]
    _serve(srv, clock, specs)
    assert len(srv.finished_jobs) == 8
    for st in srv.finished_jobs:
        assert [int(r[1]) for r in st.results] == [1, 2]
    assert be.groups and max(len(g) for g in be.groups) == 4
    for g in be.groups:
        assert len(set(g)) == len(g)
        assert len({6 if j < 6 else 8 for j in g}) == 1  # never across models
    pk = srv.packing()
    assert pk["packed_launches"] == len(be.groups)
    assert pk["requests_per_launch"] > 1.5


def test_packing_off_for_one_job_per_launch():
    clock = Clock()
    be = PackingBackend(clock)
    srv = SV.Server(be, n_slots=2, hbm_budget=1 << 30, clock=clock, group_max=1)
    specs = [SV.JobSpec(j, S.atom(6), 256, requests=2, seed=j, param_seed=0) for j in range(4)]
    _serve(srv, clock, specs)
    assert not be.groups and srv.packing()["requests_per_launch"] == 1.0
