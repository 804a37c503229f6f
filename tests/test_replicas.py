"""bench.py at N > 1: one independent replica per rank (the path does not shard), the job's rate
taken over the slowest rank.  Two ranks over gloo on CPU, as torchrun starts them (RANK,
WORLD_SIZE, MASTER_ADDR 127.0.0.1); the reference arm runs on rank 0 alone."""
import multiprocessing as mp
import os
import socket
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    assert bench.dist_env() == (ws, rank, rank)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    ms = 10.0 + 2.5 * rank  # rank 1 is the slower replica
    value, ms_max = bench.aggregate_replicas(ms, 1000, 4, ws, "cpu")
    dist.destroy_process_group()
    q.put((rank, value, ms_max))


def test_two_replicas_report_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_replica, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=180)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, ms_max in res:
        assert ms_max == 12.5
        assert value == 1000 * 4 * 2 / 12.5e-3


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    value, ms = bench.aggregate_replicas(8.0, 500, 10, 1, "cpu")
    assert ms == 8.0 and value == 500 * 10 / 8e-3


def test_reference_arm_runs_on_rank_zero_only(monkeypatch, capsys):
    sys.path.insert(0, ROOT)
    import bench
    calls = []
    monkeypatch.setattr(bench, "oracle_step_time", lambda *a, **k: calls.append(1) or (0.0, 1, (1, 1, 1)))

    class Args:
        steps, warmup, workload = 2, 3, "cart_filament_128"
    bench.reference_arm(Args(), {}, 2, 1)
    assert calls == [] and capsys.readouterr().out == ""


def test_reference_arm_line_keeps_the_bench_contract(capsys):
    """The reference arm's JSON line on rank 0: the bench keys, a cpu_baseline describing the run, an
    e2e with no host-device bytes, and a sample no larger than the workload's grid."""
    sys.path.insert(0, ROOT)
    import json
    import bench
    from searay_gb300 import workloads

    class Args:
        steps, warmup, workload = 3, 3, "cyl_kerr_64"
    vd = workloads.WORKLOADS[Args.workload]()
    bench.reference_arm(Args(), vd, 1, 0)
    d = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 3 and d["warmup"] == 3 and d["value"] > 0
    assert d["config"]["workload"] == "cyl_kerr_64"
    assert d["sample_grid"] == d["config"]["grid"] == [257, 64, 1]
    # the workload description is the one the GPU arm's line carries
    assert d["config"] == bench.config_of(Args(), vd, 1)
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["unit"] == d["unit"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def test_reference_sample_scales_radial_modes():
    """A cylindrical sample below the workload's radial size keeps the same fraction of radial modes."""
    sys.path.insert(0, ROOT)
    import bench
    from searay_gb300 import workloads
    t, P, N = bench.oracle_step_time(workloads.WORKLOADS["cyl_silica_512"](), 16)
    assert tuple(N[:3]) == (2049, 16, 1) and P == 2049 * 16 and t > 0


def test_cpu_baseline_repeats_steps_to_its_time():
    """The cpu_baseline leg repeats the oracle step until its time is reached and says so."""
    sys.path.insert(0, ROOT)
    import bench
    from searay_gb300 import workloads
    vd = workloads.WORKLOADS["cyl_kerr_64"]()
    cb, v, out = bench.cpu_baseline(vd, min_seconds=0.5, max_steps=50)
    assert cb["kind"] == "port" and cb["value"] > 0 and cb["unit"] == bench.UNIT
    steps = int(cb["sample"].split()[0])
    assert 1 < steps <= 50 and "on the full 257x64x1 grid" in cb["sample"]
    assert v["wave grid"] == vd["wave grid"] and out is None


def test_cpu_baseline_first_step_matches_the_oracle_propagator():
    """The first-step outputs the bench compares both GPU forms with are the oracle propagator's own
    outputs for one fixed step (the same medium sample, step and finish)."""
    sys.path.insert(0, ROOT)
    import bench
    from oracle import uppe_oracle as O
    from searay_gb300 import workloads
    vd = workloads.WORKLOADS["cart_filament_128"]()
    v = bench.sample_volume(vd, 16)
    _, steps, _, _, out = bench.oracle_run(v, outputs=True)
    orc = O.Oracle(v)
    dz = v["size"][2] / v["subcycles"]
    a = v["incoming wave"](orc.g.w, orc.g.x1, orc.g.x2)
    ref = orc.propagator(a, 0.0, dz, 1, dz)
    assert steps == 1 and ref[4] == 1
    errs = bench.field_metrics(*out, ref[:4])
    assert max(errs.values()) < 1e-12, errs
