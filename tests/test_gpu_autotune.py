"""The launch-shape autotuner: the first graph-replayed cycle on a mesh times the
candidate shapes of the ghost copy and the WENO5/HLL sweep and caches a choice; the
cycles that follow use it and still match the oracle (the parity tests of the stencil
suite also run on tuned shapes)."""
import numpy as np
import pytest

import oracle_lib as O
import parthenon_gb300 as pg
from parthenon_gb300 import _native as nat

pytestmark = pytest.mark.gpu


def test_tuner_records_choices_and_results_hold():
    nx, bnx, ng, ncomp = (32,) * 3, (16,) * 3, 4, 5
    mesh = pg.Mesh(nx, bnx, ng)
    state = pg.problems.burgers_state(mesh, nscalars=2, nmodes=16, kmax=6, seed=5)
    drv = pg.RK2Driver(mesh, ncomp, pg.StageConfig("burgers", "weno5", 0.8))
    drv.set_state(state)
    drv.run(3, graph=True)
    drv.stream.synchronize()
    rep = nat.tune_report()
    keys = [k for k in rep if k.startswith("burgers_dir nc=5 n=16")]
    assert keys, rep
    for k in keys + [k for k in rep if k.startswith("k_copy ncomp=5 n=16")]:
        choice, ms = rep[k]
        assert 0 <= choice < len(ms) and len(ms) in (3, 4)
        assert all(t > 0 for t in ms)
    o = O.OracleSim(nx, bnx, ng, ncomp=ncomp, physics="burgers", recon=0, cfl=0.8, prolong_in_stage=False)
    o.base()[:] = state
    o.exchange(True, 0)
    o.init_dt()
    o.run(3)
    g = drv.base.cpu().numpy()[:, :, ng:-ng, ng:-ng, ng:-ng]
    r = np.array(o.base())[:, :, ng:-ng, ng:-ng, ng:-ng]
    err = np.abs(g - r).max(axis=(0, 2, 3, 4)) / np.abs(r).max(axis=(0, 2, 3, 4))
    assert err.max() <= 1e-12, err
