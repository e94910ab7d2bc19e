"""Evaluation stage and estimator pipeline orchestration (host logic, CPU).

Mirrors the reference's EstimatorPipeline contract
(src/jaqmc/estimator/base.py:287-427): estimators run in order and see the
earlier walker statistics, ``reduce`` output is merged per step, the digest
is the NaN-skipping mean over steps merged with ``finalize_state``, and
``finalize_stats`` before any ``evaluate`` is an error.  The evaluation stage
(src/jaqmc/workflow/stage/evaluation.py:150-272) samples, estimates and writes
``[prefix_]stats.npz`` / ``[prefix_]digest.npz``.  Numerics use fakes here;
the GPU path is covered in test_gpu_vmc_api.py.
"""
import os

import numpy as np
import pytest

from jaqmc_gb300 import vmc


class _Xest:
    def init(self, data, rngs=None):
        return 0

    def evaluate_batch_walkers(self, params, bd, prev, state, rngs=None):
        x = np.asarray(bd.data.electrons, np.float64).reshape(len(bd.data.electrons), -1)[:, 0]
        return {"x": x}, state + 1

    def reduce(self, ws):
        x = ws["x"]
        return {"x": float(np.mean(x)), "x_var": float(np.var(x))}


class _Yest:
    def evaluate_batch_walkers(self, params, bd, prev, state, rngs=None):
        return {"y": 2.0 * prev["x"]}, state

    def reduce(self, ws):
        y = ws["y"]
        return {"y": float(np.mean(y)) if len(y) > 1 else float("nan")}

    def finalize_state(self, state, *, n_steps):
        return {"steps_seen": n_steps}


class _Wf:
    def batch_log_prob(self, params, data):
        return None


class _Sampler:
    """Shifts every walker by +1 per step."""

    def step(self, log_prob, data, state):
        return vmc.MoleculeData(np.asarray(data.electrons) + 1.0, data.atoms, data.charges), {"pmove": 1.0}, state + 1


def _data(b=4, n=2):
    e = np.arange(b * n * 3, dtype=np.float64).reshape(b, n, 3)
    return vmc.MoleculeData(e, np.zeros((1, 3)), np.ones(1))


def test_pipeline_order_reduce_and_digest():
    pipe = vmc.EstimatorPipeline({"x": _Xest(), "y": _Yest()})
    with pytest.raises(RuntimeError):
        pipe.finalize_stats({"x": np.zeros(2)}, {})
    state = pipe.init(_data())
    stats, state = pipe.evaluate(None, vmc.BatchedData(_data()), state)
    x0 = np.arange(4 * 6, dtype=np.float64).reshape(4, 6)[:, 0]
    assert stats["x"] == pytest.approx(x0.mean()) and stats["x_var"] == pytest.approx(x0.var())
    assert stats["y"] == pytest.approx(2 * x0.mean())
    assert state == {"x": 1, "y": None}
    dig = pipe.digest({"x": np.array([1.0, 3.0]), "x_var": np.array([0.5, np.nan]), "y": np.array([np.nan, 4.0])},
                      state, n_steps=2)
    assert dig["x"] == pytest.approx(2.0) and dig["x_var"] == pytest.approx(0.5) and dig["y"] == pytest.approx(4.0)
    assert dig["steps_seen"] == 2


def test_evaluation_stage_files_and_burn_in(tmp_path):
    pipe = vmc.EstimatorPipeline({"x": _Xest(), "y": _Yest()})
    seen = []
    stage = vmc.EvaluationStage(_Wf(), _Sampler(), pipe, iterations=5, burn_in=3, digest_step_interval=2,
                                save_dir=str(tmp_path), prefix="eval", log=lambda step, d: seen.append(step))
    digest, stacked, data, sstate, est_state = stage.run(None, _data(), 0)
    x0 = np.arange(4 * 6, dtype=np.float64).reshape(4, 6)[:, 0].mean()
    # burn-in moves the walkers by 3, then each iteration by 1 before estimating
    np.testing.assert_allclose(stacked["x"], x0 + 3 + np.arange(1, 6))
    assert sstate == 8 and est_state["x"] == 5
    assert digest["x"] == pytest.approx(x0 + 6.0) and digest["steps_seen"] == 5
    assert seen == [1, 3, 4]
    st = np.load(os.path.join(tmp_path, "eval_stats.npz"))
    dg = np.load(os.path.join(tmp_path, "eval_digest.npz"))
    assert set(st.files) == {"x", "x_var", "y"} and float(dg["x"]) == pytest.approx(x0 + 6.0)
