"""bench.py without a GPU: the JSON line of the reference arm (the reference's
own KH driver translated to C, or the oracle's restatement where the
translation is absent, timed on the host cores), its keys and values on a small
KH grid, and how a failing further leg is reported."""
import argparse
import json

import pytest


@pytest.fixture(params=["reference", "port"])
def small_baseline(request, monkeypatch, oracle_mod):
    """The reference arm on a 64x32 KH grid: the reference's own driver
    translated to C (where oracle/_ref can be built), or the oracle port."""
    import bench
    from oracle import ref

    orig = bench.cpu_baseline
    monkeypatch.setenv("OMP_NUM_THREADS", "1")
    monkeypatch.setattr(bench, "cpu_baseline",
                        lambda steps_budget_s=1.0, omp=True, nx=0, ny=0: orig(steps_budget_s=0.2, omp=False,
                                                                              nx=64, ny=32))
    if request.param == "reference":
        if not ref.buildable():
            pytest.skip("no translation of the reference here")
        orig_ref = bench.reference_cpu
        monkeypatch.setattr(bench, "reference_cpu",
                            lambda threads, budget_s=1.0, nx=0, ny=0: orig_ref(1, budget_s=0.2, nx=64, ny=32))
    else:
        monkeypatch.setattr(bench, "reference_cpu", lambda threads, budget_s=1.0, nx=0, ny=0: None)
    bench.kind_expected = request.param
    return bench


def test_reference_arm_line(small_baseline, capsys, monkeypatch):
    monkeypatch.delenv("RANK", raising=False)
    rc = small_baseline.run_reference(argparse.Namespace(gpus=1, steps=2, warmup=3))
    assert rc == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == "cell-updates/s" and line["unit"] == "cell-updates/s"
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert (line["n_gpus"], line["steps"], line["warmup"]) == (1, 2, 3)
    assert line["scaling"] == "weak" and line["vs_baseline"] is None and line["dtype"] == "f64"
    assert line["config"]["workload"] == small_baseline.WORKLOAD
    # the same config dict as the GPU arm's line, key for key
    assert line["config"] == small_baseline.headline_config(1)
    cb = line["cpu_baseline"]
    assert cb["kind"] == small_baseline.kind_expected and cb["cores"] == 1 and cb["value"] == line["value"]
    assert "64x32" in cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_other_ranks_print_nothing(small_baseline, capsys, monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")
    assert small_baseline.run_reference(argparse.Namespace(gpus=2, steps=2, warmup=3)) == 0
    assert capsys.readouterr().out == ""


def test_failing_leg_is_reported_under_its_key():
    import bench

    def boom(_):
        raise RuntimeError("leg failed")

    assert bench._leg(boom, None) == {"error": "RuntimeError: leg failed"}
    assert bench._leg(lambda a, b: a + b, 1, 2) == 3


def test_mixed_roofline_counts_binary32_u2v_as_fp32_work():
    """The FP32-mixed roofline: the u2v part of the FP64 residual moves to the
    FP32 side for the share of cells recovered in binary32, the binding
    resource is the slowest one, and achieved / frac follow from it."""
    import bench

    total, face, rest, u2v = bench._load_flops_split("flops_kh2d.txt")
    assert abs(total - (face + rest)) < 0.2 and 0 < u2v < rest
    split = (total, face, rest, u2v)
    cps = 1.0e9
    all64 = bench._mixed_roofline(cps, split, 1250.0, 78000.0, 6800.0, u2v_fp64_share=1.0)
    none64 = bench._mixed_roofline(cps, split, 1250.0, 78000.0, 6800.0, u2v_fp64_share=0.0)
    assert all64["bound"] == none64["bound"] == "fp64"
    assert all64["fp64"]["per_cell_update"] == rest
    assert abs(none64["fp64"]["per_cell_update"] - (rest - u2v)) < 1e-9
    assert abs(none64["fp32"]["per_cell_update"] - (face + u2v)) < 1e-9
    assert abs(none64["frac"] - (rest - u2v) * cps / 1.25e12) < 1e-12
    assert none64["u2v_fp64_share"] == 0.0


def test_u2v_fp64_share_follows_the_energy_test():
    """Cells with E < rho v^2 + B^2 (internal energy below kinetic plus
    magnetic) are the ones the FP32-mixed kernels recover in FP64."""
    import numpy as np

    import bench

    U = np.zeros((9, 4))
    U[4] = 1.0                       # rho
    U[0] = [0.0, 1.0, 0.0, 0.0]      # mx
    U[5] = [0.0, 0.0, 1.0, 0.1]      # Bx
    U[3] = [1.0, 1.0, 0.9, 1.0]      # E: cell 1 has E = rho v^2, cell 2 E < B^2
    assert bench._u2v_fp64_share([U]) == 0.25
    assert bench._u2v_fp64_share([U[:, :2], U[:, 2:]]) == 0.25


def test_error_report_names_the_worst_significant_variable():
    """_errors picks the largest own-norm error among the variables that hold at
    least 1e-4 of their physical scale, and names it; _member_summary names the
    ensemble member's model and grid."""
    import numpy as np

    import bench
    from openmhd_gb300.ensemble import batched_problem_set

    rng = np.random.default_rng(0)
    b = rng.uniform(0.5, 1.5, (9, 8, 8))
    b[2] *= 1e-9  # mz: below 1e-4 of the momentum scale, not significant
    a = b.copy()
    a[2] += 1e-9  # a large own-norm error in an insignificant variable is not the max
    a[6] += 1e-8
    e = bench._errors(a, b)
    assert "mz" not in e["significant_vars"] and e["max_own_norm_var"] == "by"
    assert e["max_own_norm_rel_l1_significant"] == e["own_norm_rel_l1"]["by"]
    cfgs, models = batched_problem_set(4, seed=0)
    s = bench._member_summary(1, ["ro", "by", "en", "mx"], cfgs, models)
    assert s == {"member": 1, "var": "by", "model": "kelvin_helmholtz", "ix": cfgs[1].ix, "jx": cfgs[1].jx}
