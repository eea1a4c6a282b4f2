"""E[] psi witnesses emitted by the GPU, replayed through the oracle's successor function of the
psi-restricted graph: step 0 is the restricted initial state, every later step is the successor of
the one before with the recorded emission ordinal, and a closing edge leads back into the path. A
psi that fails has no witness."""
import numpy as np
import pytest

from oracle import pyoracle
from ptctcl_gb300 import engine
from ptctcl_gb300.engine import Backend
from golden_util import load_model, verdict_rows

pytestmark = pytest.mark.gpu

SLOW = {("grc4", "E[] x0 >= 0"), ("single4", "E[] x0 <= 3"), ("single4", "E[] x0 >= 0"), ("single4", "A<> x0 >= 3")}
ROWS = [r for r in verdict_rows(kinds=(3,)) if (r[0], r[1]) not in SLOW]


def _same(a, b):
    return all(np.array_equal(np.asarray(x), np.asarray(y)) for x, y in zip(a, b))


@pytest.mark.parametrize("model,formula,kind,p,q,result", ROWS, ids=[f"{r[0]}:{r[1]}" for r in ROWS])
def test_eg_witness_replays(model, formula, kind, p, q, result):
    net = load_model(model)
    holds, tr = engine.exists_invariant_trace(net, p, Backend.Cuda)
    assert holds == result
    if not holds:
        assert tr is None
        return
    n = len(tr["ords"])
    assert n >= 1 and tr["ords"][0] == -1
    init = pyoracle.eg_initial(net, p)
    assert init is not None
    assert _same(init, (tr["locs"][0], tr["ints"][0], tr["zones"][0]))
    for i in range(1, n):
        sl, si, sz = pyoracle.eg_successors(net, p, tr["locs"][i - 1], tr["ints"][i - 1], tr["zones"][i - 1])
        k = tr["ords"][i]
        assert 0 <= k < len(sz), (i, k, len(sz))
        assert _same((sl[k], si[k], sz[k]), (tr["locs"][i], tr["ints"][i], tr["zones"][i])), i
    if tr["loop_to"] >= 0:
        sl, si, sz = pyoracle.eg_successors(net, p, tr["locs"][n - 1], tr["ints"][n - 1], tr["zones"][n - 1])
        k, j = tr["loop_ord"], tr["loop_to"]
        assert 0 <= k < len(sz) and 0 <= j < n
        assert _same((sl[k], si[k], sz[k]), (tr["locs"][j], tr["ints"][j], tr["zones"][j]))
