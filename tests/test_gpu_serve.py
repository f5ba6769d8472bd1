"""Served form: continuous batching of plume jobs under a memory budget.

* A job's result is bit for bit the same alone and in a mix of jobs that
  arrive before, with and after it, on a budget small enough that jobs wait
  for admission: its scene's arithmetic and reductions involve only its own
  data.
* Admission respects the budget and the arrival order, and every job runs
  exactly its steps.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

m = pytest.importorskip("mantaflow_gb300")
from mantaflow_gb300 import batch as mb  # noqa: E402

JOB = dict(size=(24, 28, 20), gravity=(0.0, -4e-3, 0.0), seed=77, steps=6)


def _result(srv, jid):
    return [srv.result(jid, w) for w in (mb.DENSITY, mb.VELOCITY, mb.PRESSURE)]


def test_job_alone_equals_in_mix():
    alone = mb.PlumeServer(budget_bytes=2 * 10 ** 9)
    a = alone.submit(keep=True, **JOB)
    alone.run()
    want = _result(alone, a)
    alone.close()

    others = [dict(size=(40, 40), gravity=(0.0, -2e-3, 0.0), seed=1, steps=9),
              dict(size=(20, 20, 20), gravity=(0.0, -6e-3, 0.0), seed=2, steps=4),
              dict(size=(64, 33), gravity=(0.0, -1e-3, 0.0), seed=3, steps=7),
              dict(size=(32, 24, 28), gravity=(0.0, -8e-3, 0.0), seed=4, steps=5)]
    need = max(mb.PlumeServer.job_bytes(o["size"]) for o in others + [JOB])
    mix = mb.PlumeServer(budget_bytes=2 * need + 1)  # at most two resident jobs
    ids = [mix.submit(arrival=0.0, **others[0]), mix.submit(arrival=0.0, **others[1])]
    j = mix.submit(arrival=0.02, keep=True, **JOB)
    ids += [mix.submit(arrival=0.03, **others[2]), mix.submit(arrival=0.05, **others[3])]
    st = mix.run()
    assert st["peak_bytes"] <= 2 * need + 1
    got = _result(mix, j)
    for w, g in zip(want, got):
        assert np.array_equal(w, g)
    infos = [mix.job(q) for q in ids + [j]]
    for q, info in zip(ids + [j], infos):
        assert info["admitted"] >= info["arrival"] - 1e-9
        assert info["finished"] > info["admitted"]
    assert [mix.job(q)["steps"] for q in ids] == [o["steps"] for o in others]
    ms, jobs = mix.ticks()
    assert max(jobs) <= 2 and len(ms) == st["ticks"]
    mix.close()
