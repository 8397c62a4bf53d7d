"""use_limiter = 1: the positivity flux limiter inside wenofd, instead of the
sweeping post-process (ex3_vortex_accuracy_2d/main.f90:241-329,444-530 and
its ex4/ex5/ex6 copies), against the oracle: every value equal and the
limiter counts (den_count, pre_count) identical."""
import numpy as np
import pytest

from sweeping_fd_weno_gb300 import Batch, Solver, abi, problems

pytestmark = pytest.mark.gpu

CASES = [
    ("vortex45", {}, 0),
    ("sedov2d40", {}, 30),
    ("jet", dict(nx=96, ny=24), 10),
    ("shock12", {}, 30),
]


@pytest.mark.parametrize("name,kw,steps", CASES, ids=[c[0] for c in CASES])
def test_limiter_matches_oracle(swfd, oracle_mod, name, kw, steps):
    g = Solver(problems.workload(name, use_limiter=1, **kw))
    o = oracle_mod.Oracle(problems.workload(name, use_limiter=1, **kw))
    g.init_problem()
    o.init_problem()
    if steps:
        for _ in range(steps):
            g.step()
            o.step()
    else:
        assert g.run() == o.run()
    a, b = g.state(), o.state()
    bad = ~(a == b)
    assert not bad.any(), f"{int(bad.sum())} values differ"
    assert g.time == o.time
    sg, so = g.stats(), o.stats()
    assert sg == so
    assert so["pre_count"] > 0 and so["sweep_count"] == 0


def test_batch_rejects_the_limiter_form(swfd):
    with Batch(max_slots=2, max_nx=64, max_ny=64) as b:
        with pytest.raises(abi.SwfdError):
            b.admit(problems.workload("vortex45", use_limiter=1), 0)
