"""Continuous-batching request loop for many VMC jobs on one GPU.

A *job* is one system (a neutral atom in the serving workload) with its own
FermiNet parameters, walkers, and Philox counter, all resident on the device
from the job's admission until its last request has finished.  A *request*
of a job runs ``mh_steps`` all-electron MH updates followed by the local
energy and returns the FP64 batch mean and variance of E_L (one call of the
reference's ``MCMCSampler.step`` with ``steps=mh_steps`` plus the energy
estimators and ``mean_reduce``: src/jaqmc/sampler/mcmc.py:160-199,
src/jaqmc/estimator/base.py:27-53).

Scheduling:

* jobs arrive over time and wait in an admission queue until their resident
  state (model arena + walker buffers) fits the HBM budget;
* an admitted job's requests are queued; a job has at most one request in
  flight (its walkers are state), requests of different jobs run at the same
  time on different *slots*.  A slot is a CUDA stream with its own workspace,
  so work of different jobs overlaps on the device;
* a free slot takes the oldest queued request whose electron count equals
  that of the slot's previous request (its workspace is sized for it, and a
  captured graph may exist), else the oldest request that fits; a workspace
  grows only while the budget allows it;
* requests are packed: a slot that takes a request also takes up to
  ``group_max - 1`` more queued requests of other jobs that share its model
  (same atom, configuration and parameters, hence the same electron count),
  and runs them as one launch set over their concatenated walkers
  (``qmc_mh_steps_grouped``, where each job keeps its own Philox seed and
  device counter, then one ``qmc_local_energy`` and a per-job
  ``qmc_reduce_mean_var_segments``);
* with ``use_graphs`` each (job, slot) pair's single-job request is captured
  once into a CUDA graph (the Philox counter lives in device memory and
  advances inside the graph) and replayed; the first request of a pair runs
  eagerly, and so do packed groups (their membership changes);
* completion is tracked with CUDA events and results come back through pinned
  host memory; a request's latency is completion minus submission.

A job's results depend only on its own state and counters: they are bitwise
the same whether the job runs alone or among others, packed or not, on any
slot, eagerly or from a graph.
"""
from __future__ import annotations

import collections
import time
from dataclasses import dataclass, field

import numpy as np

from . import params as P
from . import systems as S


@dataclass
class JobSpec:
    job_id: int
    mol: S.Molecule
    walkers: int
    requests: int = 1
    seed: int = 0              # walkers and Philox stream (and parameters when param_seed is None)
    arrival: float = 0.0
    param_seed: int | None = None  # parameters; jobs with equal seeds and systems share a model

    @property
    def params_seed(self) -> int:
        return self.seed if self.param_seed is None else self.param_seed


@dataclass
class Request:
    job_id: int
    index: int
    submitted: float
    start: float | None = None
    done: float | None = None
    slot: int | None = None
    graph: bool = False
    group: int = 1           # requests in the launch set (packed jobs)
    result: np.ndarray | None = None


@dataclass
class JobState:
    spec: JobSpec
    footprint: int
    request_bytes: int
    handle: object = None          # backend-owned device state
    admitted: float = 0.0
    finished: float | None = None
    issued: int = 0
    completed: int = 0
    results: list = field(default_factory=list)

    @property
    def n_electrons(self) -> int:
        return self.spec.mol.n_electrons


@dataclass
class Slot:
    index: int
    stream: object = None
    ws: object = None
    ws_bytes: int = 0
    last_n: int = -1
    request: Request | None = None               # the first request of the launch set
    group: list = field(default_factory=list)    # every request of the launch set
    event: object = None
    graphs: dict = field(default_factory=dict)


class Server:
    """The scheduler; device work goes through ``backend`` (CudaBackend on a
    GPU, or a simulated backend for testing the scheduling logic)."""

    def __init__(self, backend, n_slots: int = 8, hbm_budget: int = 150 << 30, use_graphs: bool = True,
                 clock=time.perf_counter, group_max: int = 8, group_walkers: int = 8192):
        self.backend = backend
        self.budget = int(hbm_budget)
        self.use_graphs = bool(use_graphs)
        self.group_max = int(group_max) if hasattr(backend, "run_group") else 1
        self.group_walkers = int(group_walkers)
        self.launches = 0
        self.packed_launches = 0
        self.clock = clock
        self.t0 = clock()
        self.slots = [Slot(i, backend.new_stream()) for i in range(n_slots)]
        self.pending_jobs: collections.deque[JobSpec] = collections.deque()
        self.jobs: dict[int, JobState] = {}
        self.queue: list[Request] = []
        self.finished: list[Request] = []
        self.finished_jobs: list[JobState] = []
        self.used = 0
        self.peak_used = 0

    def now(self) -> float:
        return self.clock() - self.t0

    # -- memory ----------------------------------------------------------
    def _charge(self, nbytes: int):
        self.used += nbytes
        self.peak_used = max(self.peak_used, self.used)

    # -- jobs ------------------------------------------------------------
    def arrive(self, spec: JobSpec):
        """A job arrives; it is admitted as soon as its resident state fits."""
        self.pending_jobs.append(spec)

    def _admit(self):
        while self.pending_jobs:
            spec = self.pending_jobs[0]
            fp = self.backend.job_footprint(spec)
            need = self.backend.request_bytes(spec)
            if fp + need > self.budget:
                raise MemoryError(f"job {spec.job_id} needs {fp + need} bytes, more than the budget")
            if self.used + fp > self.budget:
                return
            self.pending_jobs.popleft()
            st = JobState(spec, fp, need)
            st.handle = self.backend.create_job(spec)
            st.admitted = self.now()
            self._charge(fp)
            self.jobs[spec.job_id] = st
            self._submit_next(st)

    def _submit_next(self, st: JobState):
        if st.issued < st.spec.requests:
            self.queue.append(Request(st.spec.job_id, st.issued, self.now()))
            st.issued += 1

    def _release(self, st: JobState):
        for s in self.slots:
            s.graphs.pop(st.spec.job_id, None)
        self.backend.release_job(st.handle)
        st.handle = None
        self.used -= st.footprint
        st.finished = self.now()
        del self.jobs[st.spec.job_id]
        self.finished_jobs.append(st)

    # -- slots -----------------------------------------------------------
    def _fit(self, slot: Slot, need: int) -> bool:
        if slot.ws_bytes >= need:
            return True
        if self.used - slot.ws_bytes + need > self.budget:
            return False
        slot.graphs.clear()           # graphs bound to the old workspace
        self.backend.free_workspace(slot.ws)
        slot.ws = None
        self.used -= slot.ws_bytes
        slot.ws, slot.ws_bytes = self.backend.new_workspace(need, slot.stream), need
        self._charge(need)
        return True

    def _shrink_idle(self, need: int):
        """Free idle slots' workspaces (largest first) until ``need`` more bytes fit."""
        for s in sorted(self.slots, key=lambda s: -s.ws_bytes):
            if self.used + need <= self.budget:
                return
            if s.request is None and s.ws_bytes:
                s.graphs.clear()
                self.backend.free_workspace(s.ws)
                s.ws = None
                self.used -= s.ws_bytes
                s.ws_bytes = 0

    def _busy_jobs(self) -> set:
        return {r.job_id for s in self.slots for r in s.group}

    def _pick(self, slot: Slot):
        busy = self._busy_jobs()
        cands = [r for r in self.queue if r.job_id not in busy]
        if not cands:
            return None
        same = [r for r in cands if self.jobs[r.job_id].n_electrons == slot.last_n]
        for r in same + [r for r in cands if r not in same]:
            if self._fit(slot, self.jobs[r.job_id].request_bytes):
                return r
        # nothing fits while other slots idle on large workspaces: the oldest
        # request gets their memory
        oldest = cands[0]
        self._shrink_idle(self.jobs[oldest.job_id].request_bytes - slot.ws_bytes)
        if self._fit(slot, self.jobs[oldest.job_id].request_bytes):
            return oldest
        return None

    def _pack(self, slot: Slot, r: Request) -> list:
        """``r`` and up to group_max - 1 queued requests of other idle jobs with
        r's model, oldest first, within the walker cap; the group only if the
        slot's workspace can hold it."""
        if self.group_max <= 1:
            return [r]
        spec = self.jobs[r.job_id].spec
        key = self.backend.model_key(spec)
        busy = self._busy_jobs() | {r.job_id}
        group, specs, total = [r], [spec], spec.walkers
        for q in self.queue:
            if len(group) >= self.group_max:
                break
            st = self.jobs[q.job_id]
            if q.job_id in busy or self.backend.model_key(st.spec) != key:
                continue
            if total + st.spec.walkers > self.group_walkers:
                continue
            group.append(q)
            specs.append(st.spec)
            busy.add(q.job_id)
            total += st.spec.walkers
        if len(group) > 1 and not self._fit(slot, self.backend.group_request_bytes(specs)):
            return [r]
        return group

    def _launch(self, slot: Slot, group: list):
        r = group[0]
        st = self.jobs[r.job_id]
        jid = st.spec.job_id
        if len(group) > 1:
            self.backend.run_group([self.jobs[q.job_id].handle for q in group], slot.ws, slot.ws_bytes,
                                   slot.stream)
            self.packed_launches += 1
        else:
            g = slot.graphs.get(jid) if self.use_graphs else None
            if g is not None:
                self.backend.replay(g, slot.stream)
                r.graph = True
            else:
                self.backend.run_request(st.handle, slot.ws, slot.ws_bytes, slot.stream)
                if self.use_graphs:
                    slot.graphs[jid] = self.backend.capture(st.handle, slot.ws, slot.ws_bytes, slot.stream)
        self.launches += 1
        slot.event = self.backend.record(slot.stream)
        slot.request, slot.group, slot.last_n = r, list(group), st.n_electrons
        now = self.now()
        for q in group:
            q.start, q.slot, q.group = now, slot.index, len(group)

    def _dispatch(self):
        for slot in self.slots:
            if slot.request is not None or not self.queue:
                continue
            r = self._pick(slot)
            if r is None:
                continue
            self.queue.remove(r)
            group = self._pack(slot, r)
            for q in group[1:]:
                self.queue.remove(q)
            self._launch(slot, group)

    def _reap(self):
        for slot in self.slots:
            if slot.request is None or not self.backend.query(slot.event):
                continue
            done = self.now()
            group, slot.request, slot.group, slot.event = slot.group, None, [], None
            for r in group:
                st = self.jobs[r.job_id]
                r.result = self.backend.result(st.handle)
                r.done = done
                self.finished.append(r)
                st.results.append(r.result)
                st.completed += 1
                if st.completed == st.spec.requests:
                    self._release(st)
                else:
                    self._submit_next(st)

    def step(self):
        self._reap()
        self._admit()
        self._dispatch()

    def busy(self) -> bool:
        return bool(self.pending_jobs or self.queue or any(s.request is not None for s in self.slots))

    def packing(self) -> dict:
        """Launch sets issued, how many were packed, and requests per launch."""
        n = len(self.finished)
        return {"launches": self.launches, "packed_launches": self.packed_launches,
                "requests_per_launch": n / self.launches if self.launches else 0.0}

    def drain(self, timeout: float = 600.0, poll: float = 1e-4):
        t = self.clock()
        while self.busy():
            self.step()
            if self.clock() - t > timeout:
                raise TimeoutError("requests did not finish in time")
            if poll:
                time.sleep(poll)

    def run_arrivals(self, specs: list[JobSpec], timeout: float = 600.0, poll: float = 1e-4):
        """Serve jobs arriving ``spec.arrival`` seconds after the call (the
        specs' arrival times are rebased onto the server clock)."""
        specs = sorted(specs, key=lambda s: s.arrival)
        base = self.now()
        t_end = self.clock() + timeout
        i = 0
        while i < len(specs) or self.busy():
            now = self.now() - base
            while i < len(specs) and specs[i].arrival <= now:
                sp = specs[i]
                sp.arrival = base + sp.arrival
                self.arrive(sp)
                i += 1
            self.step()
            if self.clock() > t_end:
                raise TimeoutError("requests did not finish in time")
            if poll:
                time.sleep(poll)

    # -- statistics ------------------------------------------------------
    def request_latencies_ms(self) -> np.ndarray:
        return np.array([1e3 * (r.done - r.submitted) for r in self.finished])

    def job_latencies_ms(self) -> np.ndarray:
        return np.array([1e3 * (j.finished - j.spec.arrival) for j in self.finished_jobs])


def atom_job_specs(n_jobs: int, rate: float, seed: int = 0, requests: int = 1,
                   walker_choices=(256, 512, 1024, 2048, 4096), z_range=(2, 18),
                   param_seed: int | None = 0) -> list[JobSpec]:
    """Poisson arrivals (rate jobs/s) of neutral atoms with Z ~ U{z_range}
    (Hund's-rule spins) and walker counts ~ U(walker_choices); job j uses
    seed j for its walkers and Philox stream and ``param_seed`` for its
    parameters (None: seed j), so jobs of one element share a model."""
    rng = np.random.default_rng(seed)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_jobs)) if rate > 0 else np.zeros(n_jobs)
    specs = []
    for j in range(n_jobs):
        z = int(rng.integers(z_range[0], z_range[1] + 1))
        B = int(rng.choice(walker_choices))
        specs.append(JobSpec(j, S.atom(z), B, requests, seed=j, arrival=float(arrivals[j]), param_seed=param_seed))
    return specs


class CudaBackend:
    """Device side of the server: one qmc model per (system, configuration,
    parameter seed), shared by the jobs that use it; a request is
    qmc_mh_steps_resident + qmc_local_energy + qmc_reduce_mean_var on the
    slot's stream, a packed group qmc_mh_steps_grouped + qmc_local_energy +
    qmc_reduce_mean_var_segments over the jobs' concatenated walkers; results
    come back through pinned host memory."""

    def __init__(self, precision: str = "mixed", mh_steps: int = 20, stddev: float = 0.02, device=None,
                 config=None):
        import torch
        from . import _native
        self.torch = torch
        self.native = _native
        self.lib = _native.load()
        dev = torch.device(device or "cuda")
        if dev.index is None:
            dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        self.precision = precision
        self.mh_steps = int(mh_steps)
        self.stddev = float(stddev)
        self.config = dict(config or {})
        self._ws_sizes: dict = {}
        self._models: dict = {}  # model key -> (model, reference count)

    def cfg(self, spec: JobSpec):
        return P.FermiNetConfig(nspins=spec.mol.nspins, **self.config)

    def new_stream(self):
        return self.torch.cuda.Stream(device=self.device)

    def job_footprint(self, spec: JobSpec) -> int:
        cfg = self.cfg(spec)
        npar = P.count(P.ferminet_leaves(cfg, spec.mol.n_atoms))
        n = spec.mol.n_electrons
        # FP32 arena with transposed copies, two BF16 planes, the walker buffers
        return int(12 * npar + 4 * npar + spec.walkers * (12 * n + 16) + 4096)

    def _ws_bytes(self, spec: JobSpec, walkers: int) -> int:
        key = (spec.mol.nspins, spec.mol.n_atoms, walkers)
        if key not in self._ws_sizes:
            m = self.native.NativeFermiNet(self.cfg(spec), spec.mol.atoms, spec.mol.charges,
                                           precision=self.precision, device=self.device)
            self._ws_sizes[key] = max(int(self.lib.qmc_workspace_size(m.h, self.native.OP_MH, walkers)),
                                      int(self.lib.qmc_workspace_size(m.h, self.native.OP_LOCAL_ENERGY, walkers)))
        return self._ws_sizes[key]

    def request_bytes(self, spec: JobSpec) -> int:
        return self._ws_bytes(spec, spec.walkers)

    def group_request_bytes(self, specs) -> int:
        return self._ws_bytes(specs[0], sum(sp.walkers for sp in specs))

    def model_key(self, spec: JobSpec):
        mol = spec.mol
        return (tuple(mol.nspins), np.asarray(mol.atoms, np.float32).tobytes(),
                np.asarray(mol.charges, np.float32).tobytes(), tuple(sorted(self.config.items())), spec.params_seed)

    def _model(self, spec: JobSpec):
        key = self.model_key(spec)
        if key in self._models:
            m, refs = self._models[key]
            self._models[key] = (m, refs + 1)
            return m
        cfg = self.cfg(spec)
        m = self.native.NativeFermiNet(cfg, spec.mol.atoms, spec.mol.charges, precision=self.precision,
                                       device=self.device)
        tree = P.init_ferminet(cfg, spec.mol.n_atoms, seed=spec.params_seed)
        flat = self.torch.as_tensor(P.flatten(tree, P.ferminet_leaves(cfg, spec.mol.n_atoms)))
        m.set_params(flat.to(self.device))
        self._models[key] = (m, 1)
        return m

    def create_job(self, spec: JobSpec):
        torch = self.torch
        m = self._model(spec)
        B = spec.walkers
        x = torch.as_tensor(S.init_walkers(spec.mol, B, seed=spec.seed + 1)).to(self.device).contiguous()
        h = {
            "model": m, "spec": spec, "electrons": x,
            "log_prob": torch.empty(B, dtype=torch.float32, device=self.device),
            "accepts": torch.zeros(B, dtype=torch.int32, device=self.device),
            "e_local": torch.empty(B, dtype=torch.float32, device=self.device),
            "mean_var": torch.empty(2, dtype=torch.float64, device=self.device),
            "acc_sum": torch.empty(1, dtype=torch.float64, device=self.device),
            "counter": torch.zeros(1, dtype=torch.int64, device=self.device),
            "host": torch.empty(3, dtype=torch.float64, pin_memory=True),
        }
        # the slots' streams do not order against the default stream
        torch.cuda.current_stream(self.device).synchronize()
        return h

    def release_job(self, h):
        key = self.model_key(h["spec"])
        m, refs = self._models[key]
        if refs <= 1:
            del self._models[key]
        else:
            self._models[key] = (m, refs - 1)
        h.clear()

    def new_workspace(self, nbytes: int, stream):
        with self.torch.cuda.stream(stream):
            return self.torch.empty(nbytes, dtype=self.torch.uint8, device=self.device)

    def free_workspace(self, ws):
        pass

    def _enqueue(self, h, ws, ws_bytes, stream):
        torch, lib, check = self.torch, self.lib, self.native.check
        m, spec = h["model"], h["spec"]
        B = spec.walkers
        st = stream.cuda_stream
        h["accepts"].zero_()
        check(lib.qmc_mh_steps_resident(m.h, B, self.mh_steps, self.stddev, spec.seed, h["counter"].data_ptr(),
                                        h["electrons"].data_ptr(), h["log_prob"].data_ptr(),
                                        h["accepts"].data_ptr(), None, ws.data_ptr(), ws_bytes, st))
        check(lib.qmc_local_energy(m.h, B, h["electrons"].data_ptr(), h["e_local"].data_ptr(), None, None, None,
                                   None, ws.data_ptr(), ws_bytes, st))
        check(lib.qmc_reduce_mean_var(B, h["e_local"].data_ptr(), h["mean_var"].data_ptr(), st))
        torch.sum(h["accepts"], dim=0, keepdim=True, dtype=torch.float64, out=h["acc_sum"])
        h["host"][:2].copy_(h["mean_var"], non_blocking=True)
        h["host"][2:].copy_(h["acc_sum"], non_blocking=True)

    def run_request(self, h, ws, ws_bytes, stream):
        with self.torch.cuda.stream(stream):
            self._enqueue(h, ws, ws_bytes, stream)

    def run_group(self, hs, ws, ws_bytes, stream):
        """One launch set for the requests of jobs sharing a model: their
        walkers, counters and seeds gathered, grouped MH + local energy over
        the concatenation, per-job statistics, then everything scattered back."""
        torch, lib, check = self.torch, self.lib, self.native.check
        m = hs[0]["model"]
        Bs = [h["spec"].walkers for h in hs]
        offs = np.concatenate([[0], np.cumsum(Bs)]).astype(np.int32)
        total = int(offs[-1])
        st = stream.cuda_stream
        with torch.cuda.stream(stream):
            host = torch.empty(len(hs) * 3 + 1, dtype=torch.int64).pin_memory()
            host[:len(hs) + 1] = torch.as_tensor(offs.astype(np.int64))
            host[len(hs) + 1:2 * len(hs) + 1] = torch.as_tensor([h["spec"].seed for h in hs], dtype=torch.int64)
            tables = host.to(self.device, non_blocking=True)
            off_d = tables[:len(hs) + 1].to(torch.int32)
            seeds = tables[len(hs) + 1:2 * len(hs) + 1].contiguous()
            ctr = torch.cat([h["counter"] for h in hs])
            x = torch.cat([h["electrons"] for h in hs])
            lp = torch.empty(total, dtype=torch.float32, device=self.device)
            acc = torch.zeros(total, dtype=torch.int32, device=self.device)
            el = torch.empty(total, dtype=torch.float32, device=self.device)
            mv = torch.empty((len(hs), 2), dtype=torch.float64, device=self.device)
            check(lib.qmc_mh_steps_grouped(m.h, len(hs), off_d.data_ptr(), seeds.data_ptr(), ctr.data_ptr(), total,
                                           self.mh_steps, self.stddev, x.data_ptr(), lp.data_ptr(), acc.data_ptr(),
                                           None, ws.data_ptr(), ws_bytes, st))
            check(lib.qmc_local_energy(m.h, total, x.data_ptr(), el.data_ptr(), None, None, None, None,
                                       ws.data_ptr(), ws_bytes, st))
            check(lib.qmc_reduce_mean_var_segments(len(hs), off_d.data_ptr(), el.data_ptr(), mv.data_ptr(), st))
            for j, h in enumerate(hs):
                o, B = int(offs[j]), Bs[j]
                h["electrons"].copy_(x[o:o + B])
                h["counter"].copy_(ctr[j:j + 1])
                h["mean_var"].copy_(mv[j])
                torch.sum(acc[o:o + B], dim=0, keepdim=True, dtype=torch.float64, out=h["acc_sum"])
                h["host"][:2].copy_(h["mean_var"], non_blocking=True)
                h["host"][2:].copy_(h["acc_sum"], non_blocking=True)
            # the pinned tables stay alive until the copies that read them ran
            hs[0]["_group_tables"] = host

    def capture(self, h, ws, ws_bytes, stream):
        torch = self.torch
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(stream):
            g.capture_begin(capture_error_mode="thread_local")
            try:
                self._enqueue(h, ws, ws_bytes, stream)
            finally:
                g.capture_end()
        return g

    def replay(self, g, stream):
        with self.torch.cuda.stream(stream):
            g.replay()

    def record(self, stream):
        ev = self.torch.cuda.Event()
        ev.record(stream)
        return ev

    def query(self, ev) -> bool:
        return ev.query()

    def result(self, h) -> np.ndarray:
        """(E_L mean, E_L variance, MH acceptance fraction) of the last request."""
        v = h["host"].numpy().copy()
        v[2] /= h["spec"].walkers * self.mh_steps
        return v

    def check(self, h) -> int:
        return h["model"].check_error()
