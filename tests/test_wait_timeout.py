"""The engine's bounded idle wait (ODPX_Batch_set_wait_limit): a CTA that
finds no tile waits at most the limit, then sets the timeout flag and
returns; CTAs holding tiles never wait.  A limit of a few microseconds on a
plan with far fewer tiles than CTAs must therefore end the run with
ODPX_ERR_TIMEOUT (nothing faults or hangs), and the same plan, given its
limit back, and a new plan must then return the oracle's results."""
import pytest

import odp_gb300 as og
import oracle
from conftest import same

pytestmark = pytest.mark.gpu


def test_idle_wait_limit_reports_timeout_and_the_plan_recovers():
    n, d = 4096, 8
    adj = og.conv_edge2adjacency_general(n, og.generate_random_general(n, d, seed=41), d)
    want = oracle.aspl(adj, nodes=n)
    # one tile per level per job: two jobs keep two CTAs busy, every other
    # CTA of the persistent grid is idle from the start
    og.set_tuning(wc_log2=5, slots=2, tile_rows=n)
    try:
        b = og.Batch([og.GraphSpec(adj, nodes=n)])
    finally:
        og.set_tuning()
    assert b.kernel() == "engine"
    assert same(b.run()[0], want)                 # default limit (60 s): a normal run, captured
    b.set_wait_limit(2000)                        # 2 us
    for _ in range(2):
        with pytest.raises(og.ODPError) as e:
            b.run()
        assert e.value.code == og.ERR_TIMEOUT
    b.set_wait_limit(60 * 10 ** 9)
    assert same(b.run()[0], want)
    assert same(b.run()[0], want)
    b.close()
    fresh = og.Batch([og.GraphSpec(adj, nodes=n)])
    assert same(fresh.run()[0], want)
    fresh.close()
