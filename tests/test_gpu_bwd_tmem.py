"""The one-hot backward with hi + lo operands keeps its A tiles in TMEM by
default (tcgen05.st, MMAs reading A from tensor memory); SDCA_TC_BWD_SMEM_A=1
keeps them in shared memory.  Both must reach the same optima: the dual
form's exact max-norm checks and the tensor-core form's gradient run
through this kernel.  The switch is read once per process, so each setting
runs in a child process."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from superdca_gb300 import Engine, FORM_DUAL, FORM_TC, synthetic
st, _, _ = synthetic.workload("tree-3000x10000", seed=5, N=600, L=3000)
N, L = st.shape
w = np.ones(N)
loci = np.arange(0, L, L // 24)[:24]
out = {}
for name, form in (("dual", FORM_DUAL), ("tc", FORM_TC)):
    with Engine(N, L, batch=8, form=form) as E:
        E.set_alignment(st, w)
        res = E.solve(loci, want_x=True)
        np.save(sys.argv[2] + "_" + name + ".npy", res.x)
        out[name] = dict(f=res.f.tolist(), status=res.status.tolist(), it=res.iterations.tolist(),
                         scores=np.nan_to_num(res.scores).tolist())
print(json.dumps(out))
"""


def _run(tmp_path, tag, smem_a):
    env = dict(os.environ)
    env.pop("SDCA_TC_BWD_SMEM_A", None)
    if smem_a:
        env["SDCA_TC_BWD_SMEM_A"] = "1"
    prefix = str(tmp_path / tag)
    out = subprocess.run([sys.executable, "-c", CHILD, ROOT, prefix], env=env, capture_output=True, text=True,
                         timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    res = json.loads(out.stdout.strip().splitlines()[-1])
    for name in res:
        res[name]["x"] = np.load(prefix + "_" + name + ".npy")
    return res


def test_backward_a_in_tmem_matches_shared_memory(tmp_path, engine_lib, oracle_mod):
    from superdca_gb300 import synthetic

    tm = _run(tmp_path, "tmem", False)
    sm = _run(tmp_path, "smem", True)
    st, _, _ = synthetic.workload("tree-3000x10000", seed=5, N=600, L=3000)
    N, L = st.shape
    w = np.ones(N)
    from superdca_gb300 import Engine

    with Engine(N, L) as E:
        E.set_alignment(st, w)
        lh, lJ, _ = E.lambdas()
    P = oracle_mod.Problem(st, w, lh, lJ)
    loci = np.arange(0, L, L // 24)[:24]
    for name in ("dual", "tc"):
        a, b = tm[name], sm[name]
        assert set(a["status"]) == {0} and set(b["status"]) == {0}, (name, a["status"], b["status"])
        np.testing.assert_allclose(a["f"], b["f"], rtol=1e-6, err_msg=name)
        np.testing.assert_allclose(np.array(a["scores"]), np.array(b["scores"]), atol=1e-4, err_msg=name)
        # the TMEM path's solutions against the FP64 oracle: objective and stop test
        for k in (0, 7, 23):
            f64, g64 = P.objective(int(loci[k]), a["x"][k])
            assert a["f"][k] == pytest.approx(f64, rel=1e-6), (name, k)
            assert np.abs(g64).max() < 1.05e-3, (name, k, np.abs(g64).max())
