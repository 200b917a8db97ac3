"""bench.py's host logic on CPU: the multi-replica path (gloo, world size 2)
and the clock summary of the bench line.

The solve path does not shard, so `bench.py --gpus N` runs N replicas: each
rank solves its own copy, the ranks meet at barriers around the timed region,
the time reported is the maximum over ranks, and rank 0 alone prints the JSON
line (the reference arm runs on rank 0 only).  These tests run that host
logic as two gloo processes on 127.0.0.1 without a GPU."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _env(**extra):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", CUDA_VISIBLE_DEVICES="")
    env.update({k: str(v) for k, v in extra.items()})
    return env


CHILD = r"""
import json, sys
sys.path.insert(0, {root!r})
import bench
rank, world, dist = bench.dist_init(2)
assert world == 2 and dist is not None and dist.get_backend() == "gloo"
bench.barrier(dist)
m = bench.max_over_ranks(0.25 + rank, dist)
bench.barrier(dist)
print(json.dumps({{"rank": rank, "max": m}}))
dist.destroy_process_group()
"""


def test_max_over_ranks_two_gloo_ranks():
    """dist_init joins the gloo group, barrier passes, and every rank gets the
    maximum of the per-rank times."""
    port = _free_port()
    procs = [subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], cwd=ROOT, text=True,
                              stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                              env=_env(WORLD_SIZE=2, RANK=r, LOCAL_RANK=r, MASTER_PORT=port))
             for r in range(2)]
    outs = []
    try:
        for p in procs:
            outs.append(p.communicate(timeout=180))
    finally:
        for p in procs:
            if p.poll() is None:
                p.kill()
    for p, (_, err) in zip(procs, outs):
        assert p.returncode == 0, err[-2000:]
    res = sorted((json.loads(o.strip().splitlines()[-1]) for o, _ in outs), key=lambda d: d["rank"])
    assert [d["rank"] for d in res] == [0, 1]
    assert all(d["max"] == 1.25 for d in res)


def test_max_over_ranks_without_group_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(0.5, None) == 0.5
    bench.barrier(None)


def test_reference_arm_under_torchrun_prints_once():
    """`bench.py --impl reference --gpus 2` under torch.distributed.run: both
    ranks exit 0, rank 0 alone prints one JSON line (16^3 grid, one step)."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--grid", "16"]
    out = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600, env=_env())
    assert out.returncode == 0, out.stderr[-3000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.lstrip().startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["steps"] == 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["value"] > 0


def test_clock_summary_parses_each_sample_whole():
    """The bench line's clocks: median SM clock over loaded samples, the
    maximum clock, throttle reasons seen active; an [N/A] field drops only
    its own value (no misaligned clock/power pairs)."""
    sys.path.insert(0, ROOT)
    import bench
    lines = [
        "0, 1965, 2070, 120.5, 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070, [N/A], 0x0, Not Active, Not Active, Not Active, Not Active",
        "0, 2070, 2070, 790.1, 0x4, Not Active, Not Active, Not Active, Active",
        "0, 2055, 2070, 805.0, 0x0, Not Active, Not Active, Not Active, Not Active",
        "garbage line",
    ]
    s = bench.summarize_clocks(lines)
    assert s["samples"] == 4
    assert s["sm_mhz"] == 2062.5  # median of the two samples above 300 W
    assert s["sm_max_mhz"] == 2070.0 and s["power_w_max"] == 805.0
    assert s["reasons"] == ["sw_power_cap"]
    idle = bench.summarize_clocks(["0, 1200, 2070, 90.0, 0x0, Not Active, Active, Not Active, Not Active"])
    assert idle["sm_mhz"] == 1200.0 and idle["reasons"] == ["hw_thermal_slowdown"]
    assert bench.summarize_clocks([])["reasons"] == ["no samples"]
