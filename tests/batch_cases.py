"""Small batched-likelihood workloads shared by the CPU and GPU tests."""
import numpy as np

from xpsi_gb300 import batch as BT
from xpsi_gb300 import synthetic as SY


def small_num4d(V=4, seed=7):
    """A reduced copy of the full-size plain configuration (two Num4D hot
    regions, one with an omitted crescent) that the oracle runs in seconds;
    counts drawn from the oracle's model of the first vector."""
    from oracle import pipeline as OP
    m = SY.config2_model(K=60, q=24, num_energies=24, sqrt_num_cells=12, num_leaves=24,
                         num_rays=64, max_sqrt_num_cells=24, table_shape=(10, 8, 16, 60))
    rng = np.random.default_rng(seed)
    params = np.array([SY.prior_vector(rng) for _ in range(V)])
    P = BT.prepare(m, params)
    _, _, stages = OP.loglike(m, P, return_stages=True)
    SY.attach_data(m, [stages[0]["folded"], stages[1]["folded"]], P.shifts[0])
    return m, params


def small_blackbody(V=3, seed=11):
    """Blackbody hot region of the small plain configuration's kind."""
    from oracle import pipeline as OP
    w = SY.config1_workload(n_channels=50, n_inputs=20, n_energies=24)
    m = BT.Model(regions=[BT.HotRegionSpec(atm_ext=1, sqrt_num_cells=12, min_sqrt_num_cells=8,
                                           max_sqrt_num_cells=24, num_leaves=24, num_rays=64)],
                 instrument=BT.Instrument(w["matrix"], w["input_edges"]),
                 data=BT.Data(counts=np.zeros((50, 32), np.int32),
                              phase_edges=w["phase_edges"], exposure=w["exposure"]),
                 num_energies=24)
    rng = np.random.default_rng(seed)
    rows = []
    for v in range(V):
        rows.append([rng.uniform(1.2, 2.0), rng.uniform(10.0, 14.0), rng.uniform(200, 600),
                     rng.uniform(0.1, 0.9), 1.0, rng.uniform(0.2, 2.9), rng.uniform(0.05, 0.4),
                     rng.uniform(5.9, 6.4), rng.uniform(0, 1)])
    params = np.array(rows)
    P = BT.prepare(m, params)
    _, _, stages = OP.loglike(m, P, return_stages=True)
    SY.attach_data(m, [stages[0]["folded"]], P.shifts[0])
    return m, params


def small_elsewhere(V=3, seed=13, num4d=False):
    """A hot region (blackbody, or the small Num4D table) plus a blackbody
    elsewhere (closed mesh of 12 x 12 cells, 48 rays); counts drawn from the
    oracle's model of the first vector."""
    from oracle import pipeline as OP
    w = SY.config1_workload(n_channels=50, n_inputs=20, n_energies=24)
    atm = SY.num4d_table(shape=(10, 8, 16, 60)) if num4d else None
    m = BT.Model(regions=[BT.HotRegionSpec(atm_ext=2 if num4d else 1, sqrt_num_cells=12,
                                           min_sqrt_num_cells=8, max_sqrt_num_cells=24,
                                           num_leaves=24, num_rays=64)],
                 instrument=BT.Instrument(w["matrix"], w["input_edges"]),
                 data=BT.Data(counts=np.zeros((50, 32), np.int32),
                              phase_edges=w["phase_edges"], exposure=w["exposure"]),
                 num_energies=24, atmosphere=atm,
                 elsewhere=BT.ElsewhereSpec(sqrt_num_cells=12, num_rays=48))
    rng = np.random.default_rng(seed)
    rows = []
    for v in range(V):
        rows.append([rng.uniform(1.2, 2.0), rng.uniform(10.0, 14.0), rng.uniform(200, 600),
                     rng.uniform(0.1, 0.9), 1.0, rng.uniform(0.2, 2.9), rng.uniform(0.05, 0.4),
                     rng.uniform(6.0, 6.4), rng.uniform(0, 1), rng.uniform(5.6, 5.95)])
    params = np.array(rows)
    P = BT.prepare(m, params)
    _, _, stages = OP.loglike(m, P, return_stages=True)
    SY.attach_data(m, [stages[0]["folded"]], P.shifts[0])
    return m, params
