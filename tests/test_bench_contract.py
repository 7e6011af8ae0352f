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
