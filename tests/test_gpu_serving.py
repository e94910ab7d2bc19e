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
