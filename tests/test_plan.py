"""Host-side symbolic analysis of the preconditioner (no GPU).

`iemic_analyse_pattern` builds the nested-dissection plan the GPU factorisation
uses from the engine's land mask and J's CSR pattern, checks its offsets and
maps, and reports its sizes. The oracle's independent restatement of the same
ordering (oracle/multifrontal.py) must give the same elimination tree: front
count, reduced unknowns, factor entries, dense front storage and flops.
"""
import numpy as np
import pytest

import oracle
from oracle import multifrontal as MF
from helpers import box_case, global_case


def _c2():
    from iemic import workloads as W
    cfg = W.global_96x38x12()
    return cfg, W.seeded_global_mask(cfg, 0), None


CASES = {"box": box_case, "glob24": global_case, "global_96x38x12": _c2}


def _analyse(name):
    from iemic.ocean import analyse_pattern
    cfg, lm, frc = CASES[name]()
    o = oracle.Oracle(cfg, lm)
    rp, ci = o.graph()
    landm = o.landm()
    return cfg, landm, rp, ci, analyse_pattern(cfg, landm, rp, ci)


@pytest.mark.parametrize("name", sorted(CASES))
def test_plan_matches_oracle_ordering(name):
    cfg, landm, rp, ci, info = _analyse(name)
    P = MF.Plan(landm, cfg["n"], cfg["m"], cfg["l"], cfg["periodic"])
    nf = np.array([nd["nf"] for nd in P.nodes], dtype=np.int64)
    nb = np.array([len(nd["B"]) for nd in P.nodes], dtype=np.int64)
    assert info["unknowns"] == 6 * cfg["n"] * cfg["m"] * cfg["l"]
    assert info["fronts"] == len(P.nodes)
    assert info["reduced_unknowns"] == nf.sum()
    assert info["factor_entries"] == (nf * nf + 2 * nf * nb).sum()
    assert info["front_entries"] == ((nf + nb) ** 2).sum()
    assert info["factor_flops"] == pytest.approx(P.flops, rel=1e-12)
    # the reused storage is smaller than all dense fronts together
    assert info["work_entries"] <= info["front_entries"]
    assert info["contrib_entries"] <= 3 * info["front_entries"]


def test_plan_of_the_bench_workload():
    """Known answer: the 96x38x12 seeded ocean's plan as GB300 reports it."""
    *_, info = _analyse("global_96x38x12")
    assert (info["fronts"], info["levels"], info["reduced_unknowns"]) == (1023, 10, 143043)
    assert (info["factor_entries"], info["front_entries"]) == (373760857, 1092243221)
    assert (info["work_entries"], info["contrib_entries"]) == (193120330, 236080852)


def test_bad_pattern_is_rejected():
    from iemic import IemicError
    from iemic.ocean import analyse_pattern
    cfg, landm, rp, ci, _ = _analyse("box")
    bad = ci.copy()
    bad[7] = 6 * cfg["n"] * cfg["m"] * cfg["l"]   # a column past the last unknown
    with pytest.raises(IemicError):
        analyse_pattern(cfg, landm, rp, bad)
    bad_rp = rp.copy()
    bad_rp[5], bad_rp[6] = bad_rp[6], bad_rp[5] + 1   # row pointers that decrease
    with pytest.raises(IemicError):
        analyse_pattern(cfg, landm, bad_rp, ci)
