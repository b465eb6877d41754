"""The autotuner (electrodrive_gb300.fmm3d.autotune, following the
reference's electrodrive/fmm3d/autotune.py:92-849): the reference's dry-run
default, size buckets and JSON cache records (host logic, CPU), and on the
GPU a real search over configs and launch shapes whose result is stored
and reused by the next call on the same machine and bucket."""
import json

import pytest
import torch


def test_dry_run_returns_the_base_config_and_buckets_are_powers_of_two():
    from electrodrive_gb300.fmm3d import FmmConfig
    from electrodrive_gb300.fmm3d.autotune import autotune_for_problem, bucket_problem_size

    cfg = FmmConfig(expansion_order=6, leaf_size=32)
    res = autotune_for_problem(cfg, 5000)
    assert res.config is cfg and res.metrics["mode"] == 0.0 and res.launch == {}
    assert [bucket_problem_size(n) for n in (0, 1, 2, 3, 1000, 1024, 1025)] == [1, 1, 2, 4, 1024, 1024, 2048]
    with pytest.raises(ValueError):
        autotune_for_problem(cfg, 0)


def test_cache_records_are_filtered_by_machine_bucket_kind_signature_and_error(tmp_path, monkeypatch):
    from electrodrive_gb300.fmm3d import autotune as at

    path = tmp_path / "tune.json"
    monkeypatch.setenv(at.AUTOTUNE_CACHE_ENV_VAR, str(path))
    assert at.cache_path() == path and at.load_best("m", 1024, 1e-2) is None
    rec = lambda t, e, **kw: dict({"fingerprint": "m", "problem_size_bucket": 1024, "kind": "fmm",
                                   "config": {"expansion_order": 6, "precision": "mixed"}, "launch": {"near_overlap": 0},
                                   "metrics": {"wall_time_s": t, "rel_l2_error": e}}, **kw)
    at.append_record(rec(2.0, 1e-3))
    at.append_record(rec(1.0, 5e-2))                      # too inaccurate
    at.append_record(rec(0.5, 1e-3, fingerprint="other"))  # another machine
    at.append_record(rec(0.7, 1e-3, problem_size_bucket=2048))
    at.append_record(rec(1.5, 1e-3, kind="inner_fp32", signature="s"))
    assert len(json.loads(path.read_text())["records"]) == 5
    best = at.load_best("m", 1024, 1e-2)
    assert best["metrics"]["wall_time_s"] == 2.0 and best["launch"] == {"near_overlap": 0}
    assert at.load_best("m", 1024, 1e-2, kind="inner_fp32", signature="s")["metrics"]["wall_time_s"] == 1.5
    assert at.load_best("m", 1024, 1e-2, kind="inner_fp32", signature="t") is None
    assert at.load_best("m", 1024, 1e-2, precision="double") is None


@pytest.mark.gpu
def test_search_stores_its_choice_and_the_next_call_reuses_it(cuda_lib, tmp_path, monkeypatch):
    from electrodrive_gb300.fmm3d import FmmConfig
    from electrodrive_gb300.fmm3d import autotune as at

    monkeypatch.setenv(at.AUTOTUNE_CACHE_ENV_VAR, str(tmp_path / "tune.json"))
    cfg = FmmConfig(expansion_order=6, leaf_size=64)
    res = at.autotune_for_problem(cfg, 30000, dry_run=False, target_rel_error=1e-4, max_trials=8)
    assert res.metrics.get("from_cache") is None and res.metrics["rel_l2_error"] <= 1e-4
    assert res.launch.get("near_overlap") in (0, 1)
    again = at.autotune_for_problem(cfg, 30000, dry_run=False, target_rel_error=1e-4, max_trials=8)
    assert again.metrics["from_cache"] == 1.0
    assert at.cfg_to_dict(again.config) == at.cfg_to_dict(res.config) and again.launch == res.launch


@pytest.mark.gpu
def test_inner_operator_choice_is_cached_and_rechecked(cuda_lib, tmp_path, monkeypatch):
    from electrodrive_gb300.core.bem import assemble_system, autotune_inner_operator
    from electrodrive_gb300.core.bem_mesh import torus_mesh
    from electrodrive_gb300.fmm3d import autotune as at

    monkeypatch.setenv(at.AUTOTUNE_CACHE_ENV_VAR, str(tmp_path / "tune.json"))
    spec = dict(conductors=[dict(type="torus", major_radius=1.0, minor_radius=0.35, potential=1.0)],
                charges=[dict(type="point", q=1.0, pos=[1.6, 0.3, 0.2])])
    S = assemble_system(torus_mesh(1.0, 0.35, 80, 32), spec, kind="fmm", dtypes=(torch.float64, torch.float32),
                        near=True)
    args = (S["ops"][torch.float64], S["centroids"], S["areas"], S["self_corr"])
    op, trials = autotune_inner_operator(*args, near=S["ops"][torch.float32].near, orders=(8, 6))
    assert len(trials) == 4 and not any(t.get("from_cache") for t in trials)
    op2, trials2 = autotune_inner_operator(*args, near=S["ops"][torch.float32].near, orders=(8, 6))
    assert len(trials2) == 1 and trials2[0]["from_cache"] and trials2[0]["rel_error"] <= 3e-7
    assert op2.base.plan.info.expansion_order == op.base.plan.info.expansion_order
    assert op2.base.plan.get_launch() == op.base.plan.get_launch()


def test_select_trial_prefers_accuracy_among_equally_fast():
    from electrodrive_gb300.fmm3d.autotune import select_trial

    trials = [dict(name="a", ms=10.0, rel_error=2.9e-7), dict(name="b", ms=10.4, rel_error=1.7e-7),
              dict(name="c", ms=12.0, rel_error=1.0e-7), dict(name="d", ms=9.0, rel_error=5e-7)]
    # d is fastest but misses the bound; b is within 5% of a and more accurate; c is too slow
    assert select_trial(trials, 3e-7)["name"] == "b"
    assert select_trial(trials, 3e-7, time_slack=0.0)["name"] == "a"
    assert select_trial(trials, 1e-8) is None
    # with the inner tolerance the error costs iterations: cost = ms / (1 - err / tol)
    # a: 10 / (1 - 0.967) = 300, b: 10.4 / (1 - 0.567) = 24, c: 12 / (1 - 0.333) = 18
    assert select_trial(trials, 3e-7, inner_tol=3e-7)["name"] == "c"
    assert select_trial(trials, 3e-7, inner_tol=1e-5)["name"] == "a"  # a loose floor: speed decides
