"""The serving loop on the GPU: a job's results are bitwise the same alone and
in a mix with other jobs (tolerance: exact equality of the FP64 mean and
variance and of the acceptance count), from captured graphs and eagerly, and
equal to the plain qmc_mh_steps + qmc_local_energy path with the same counter.
"""
import numpy as np
import pytest
import torch

from jaqmc_gb300 import _native
from jaqmc_gb300 import serving as SV
from jaqmc_gb300 import systems as S

pytestmark = pytest.mark.gpu

MIX = [(2, 256), (6, 512), (10, 256), (18, 256), (6, 256)]


def _specs(requests=3):
    return [SV.JobSpec(j, S.atom(z), B, requests=requests, seed=j) for j, (z, B) in enumerate(MIX)]


def _serve(specs, n_slots, use_graphs=True):
    srv = SV.Server(SV.CudaBackend(precision="mixed"), n_slots=n_slots, hbm_budget=40 << 30,
                    use_graphs=use_graphs)
    for sp in specs:
        srv.arrive(sp)
    srv.drain(timeout=300)
    return srv, {st.spec.job_id: np.stack(st.results) for st in srv.finished_jobs}


def test_alone_equals_mix(cuda_device):
    srv, mix = _serve(_specs(), n_slots=3)
    assert len(mix) == len(MIX)
    assert any(r.graph for r in srv.finished)
    for j in (0, 3, 4):
        _, alone = _serve([_specs()[j]], n_slots=1)
        np.testing.assert_array_equal(alone[j], mix[j])
    for j, res in mix.items():
        assert np.all(np.isfinite(res[:, :2]))
        assert np.all((res[:, 2] > 0.05) & (res[:, 2] < 1.0)), res


def test_graphs_equal_eager(cuda_device):
    _, g = _serve(_specs(2), n_slots=2, use_graphs=True)
    _, e = _serve(_specs(2), n_slots=2, use_graphs=False)
    for j in g:
        np.testing.assert_array_equal(g[j], e[j])


def test_resident_counter_matches_host_counter(cuda_device):
    spec = _specs(2)[1]
    _, res = _serve([spec], n_slots=1)
    res = res[spec.job_id]
    be = SV.CudaBackend(precision="mixed")
    h = be.create_job(spec)
    m, x = h["model"], h["electrons"]
    for r in range(2):
        m.mh_steps(x, 20, 0.02, spec.seed, 20 * r)
        el = m.local_energy(x)["e_local"]
        mv = _native.reduce_mean_var(el).cpu().numpy()
        np.testing.assert_array_equal(mv, res[r, :2])


def test_poisson_stream(cuda_device):
    specs = SV.atom_job_specs(6, rate=50.0, seed=1, requests=2, walker_choices=(256, 512))
    srv = SV.Server(SV.CudaBackend(precision="mixed"), n_slots=4, hbm_budget=40 << 30)
    srv.run_arrivals(specs, timeout=300)
    assert len(srv.finished_jobs) == 6
    lat = srv.request_latencies_ms()
    assert lat.shape == (12,) and np.all(lat > 0)
    for st in srv.finished_jobs:
        assert st.spec.mol.n_electrons == sum(st.spec.mol.nspins)
        assert st.handle is None
    torch.cuda.synchronize()


def test_packed_requests_equal_alone(cuda_device):
    """Jobs sharing a model (carbon, parameters seed 0) packed into grouped
    launches give bitwise the results of each job served alone."""
    specs = [SV.JobSpec(j, S.atom(6), B, requests=3, seed=j, param_seed=0)
             for j, B in enumerate((256, 512, 256, 384))]
    srv = SV.Server(SV.CudaBackend(precision="mixed"), n_slots=1, hbm_budget=40 << 30, group_max=4)
    for sp in specs:
        srv.arrive(sp)
    srv.drain(timeout=300)
    packed = {st.spec.job_id: np.stack(st.results) for st in srv.finished_jobs}
    assert srv.packing()["packed_launches"] > 0
    assert max(r.group for r in srv.finished) > 1
    for sp in specs:
        _, alone = _serve([SV.JobSpec(sp.job_id, sp.mol, sp.walkers, requests=3, seed=sp.seed, param_seed=0)],
                          n_slots=1)
        np.testing.assert_array_equal(alone[sp.job_id], packed[sp.job_id])


def test_grouped_mh_equals_per_job_calls(cuda_device):
    """qmc_mh_steps_grouped over two jobs' concatenated walkers moves each
    job's walkers exactly as qmc_mh_steps_resident on that job alone."""
    be = SV.CudaBackend(precision="fp32")
    specs = [SV.JobSpec(j, S.atom(4), B, seed=10 + j, param_seed=0) for j, B in enumerate((128, 200))]
    hs = [be.create_job(sp) for sp in specs]
    m, lib = hs[0]["model"], be.lib
    x0 = [h["electrons"].clone() for h in hs]
    ws_bytes = be.group_request_bytes(specs)
    ws = torch.empty(ws_bytes, dtype=torch.uint8, device=cuda_device)
    offs = torch.tensor([0, 128, 328], dtype=torch.int32, device=cuda_device)
    seeds = torch.tensor([10, 11], dtype=torch.int64, device=cuda_device)
    ctr = torch.tensor([5, 9], dtype=torch.int64, device=cuda_device)
    x = torch.cat(x0)
    lp = torch.empty(328, dtype=torch.float32, device=cuda_device)
    acc = torch.zeros(328, dtype=torch.int32, device=cuda_device)
    _native.check(lib.qmc_mh_steps_grouped(m.h, 2, offs.data_ptr(), seeds.data_ptr(), ctr.data_ptr(), 328, 4, 0.05,
                                           x.data_ptr(), lp.data_ptr(), acc.data_ptr(), None, ws.data_ptr(),
                                           ws_bytes, 0))
    for j, (o, B, c0) in enumerate(((0, 128, 5), (128, 200, 9))):
        xe = x0[j].clone()
        lpe = torch.empty(B, dtype=torch.float32, device=cuda_device)
        acce = torch.zeros(B, dtype=torch.int32, device=cuda_device)
        ce = torch.tensor([c0], dtype=torch.int64, device=cuda_device)
        m.mh_steps_resident(xe, 4, 0.05, 10 + j, ce, lpe, acce)
        torch.cuda.synchronize()
        assert torch.equal(xe, x[o:o + B])
        assert torch.equal(lpe, lp[o:o + B])
        assert torch.equal(acce, acc[o:o + B])
        assert int(ce.item()) == int(ctr[j].item()) == c0 + 4
