"""bench.py's reference arm prints one JSON line with the contract's keys (no GPU: the oracle's
timed samples are replaced by a stand-in that returns fixed timings), on the same workload, metric
and config as the GPU arm."""
import json

import bench


def test_reference_line_carries_the_contract(monkeypatch, capsys):
    info = dict(extrapolated=True, threads=4, scgd0_sampled_fraction=0.1, scgd0_sample_s=0.2,
                scgd0_sample="stand-in scGD0 sample", ladder_sampled_fraction=0.1, ladder_sample_s=0.3,
                ladder_sample="stand-in ladder sample")
    monkeypatch.setattr(bench, "cpu_samples", lambda s, T, sigma, mu: (2.0, 3.0, 4, info))
    args = type("A", (), dict(steps=2, warmup=1))()
    bench.run_reference(args, 1, 0, 0)
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in line, key
    assert line["impl"] == "reference" and line["metric"] == bench.METRIC and line["higher_is_better"] is False
    expect = 2.0 * bench.FP64_SCGD0_ITERS + 3.0 * bench.FP64_LADDER_APPLIES
    assert abs(line["value"] - expect) < 1e-12 and abs(line["ms_per_step"] - 1e3 * expect) < 1e-9
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["cores"] == 4 and cb["kind"] == "port" and cb["sample"]
    # a sampled and scaled baseline says so, with the fractions and the measured seconds
    assert cb["extrapolated"] is True and cb["scgd0_sampled_fraction"] == 0.1 and cb["ladder_sample_s"] == 0.3
    assert line["e2e"] == dict(value=line["value"], unit="s", h2d_bytes_per_step=0, d2h_bytes_per_step=0)
    s, _, _, _ = bench.workload()
    assert line["config"] == json.loads(json.dumps(bench.bench_config(s, 1)))
    assert line["config"]["workload"].startswith("3-band cubic t2g")


def test_other_ranks_print_nothing(capsys):
    args = type("A", (), dict(steps=1, warmup=0))()
    bench.run_reference(args, 2, 1, 1)
    assert capsys.readouterr().out == ""
