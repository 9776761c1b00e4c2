"""bench.py's multi-rank host logic on CPU: world size 2 over gloo on
127.0.0.1, launched the way a multi-GPU bench run is (torch.distributed.run).

The path shards as replicas only, so the ranks exchange nothing but the timing
reductions and the final barrier; these run here without a GPU.  The reference
arm is the oracle's CPU design iteration: rank 0 alone runs it and prints the
one JSON line, the other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys
import textwrap

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=timeout)


def _json_lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def test_rank_reductions_gloo(tmp_path):
    """max/sum over ranks and the barrier, as the bench's timed region uses them."""
    script = tmp_path / "ranks.py"
    script.write_text(textwrap.dedent(f"""
        import json, sys
        sys.path.insert(0, {ROOT!r})
        import bench
        world, rank, local, pg = bench.dist_setup()
        assert pg is not None and world == 2 and local == rank
        bench.barrier(pg)
        mx = bench.max_over_ranks(pg, 1.5 + rank)
        sm = bench.sum_over_ranks(pg, 1.5 + rank)
        with open({str(tmp_path)!r} + f"/rank{{rank}}.json", "w") as f:
            json.dump({{"world": world, "max": mx, "sum": sm}}, f)
        pg.barrier()
        pg.destroy_process_group()
    """))
    r = _torchrun([str(script)], timeout=120)
    assert r.returncode == 0, r.stderr[-2000:]
    for rank in (0, 1):
        got = json.loads((tmp_path / f"rank{rank}.json").read_text())
        assert got == {"world": 2, "max": 2.5, "sum": 4.0}, (rank, got)


def test_reference_arm_two_ranks():
    """Rank 0 prints one reference line on the host cores; rank 1 prints none."""
    r = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--nx", "12", "--ny", "6",
                   "--nz", "6", "--steps", "2", "--warmup", "3"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _json_lines(r.stdout)
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["metric"] == "design_iters_per_s" and line["unit"] == "design_iters/s"
    assert line["steps"] == 2 and len(line["cg_iterations"]) == 2
    assert line["value"] > 0 and abs(line["ms_per_step"] - 1e3 / line["value"]) < 1e-6
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["value"] == line["value"]
    # torchrun exports OMP_NUM_THREADS=1; the CPU arm still uses every host core
    # (one when the oracle was built without OpenMP).
    from oracle.oracle import OracleLib
    import bench
    port = OracleLib("port")
    old = port.threads()
    port.set_threads(2)
    openmp = port.threads() == 2
    port.set_threads(old)
    assert cb["cores"] == (bench.host_cores() if openmp else 1), cb


def test_reference_arm_secondary_workloads_unavailable():
    """The secondary workloads have no CPU reference arm: one unavailable line, exit 0."""
    for w in ("batch", "homog", "serve"):
        r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", w],
                           cwd=ROOT, capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr[-2000:]
        lines = _json_lines(r.stdout)
        assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["unavailable"]
