"""bench.py's host side on the CPU: the reference arm's JSON line carries every key of the
benchmark contract (run on a 2x2x2 crystal instead of the 1024-electron workload), the
nvidia-smi clock samples are parsed into the `clocks` object, the algorithmic work of
the roofline is (32/3) n^3 real flops per window-pole solve, and the timed legs take the
slowest of two gloo ranks."""
import json
import types

import numpy as np

KEYS = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
        "vs_baseline", "dtype", "data", "config", "e2e", "cpu_baseline")


def test_reference_arm_line(monkeypatch, capsys):
    import bench
    from lresdft_gb300 import system
    cr = system.jittered_h2((2, 2, 2), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=0)
    seen = {}

    def small_system(cells=8, assembly="native"):
        seen["assembly"] = assembly
        return cr, system.LCAOBasis(cr, assembly=assembly)

    monkeypatch.setattr(bench, "build_system", small_system)
    bench.run_reference(types.SimpleNamespace(steps=1, warmup=3, scf_iters=3, cpu_scf=True))
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert seen["assembly"] == "scipy"          # the reference's own basis assembly
    assert all(k in line for k in KEYS) and line["impl"] == "reference"
    assert line["value"] > 0 and line["higher_is_better"] is True and line["vs_baseline"] is None
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["cpu_baseline"]["value"] == line["value"] == line["e2e"]["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert "workload" in line["config"]
    scf = line["cpu_baseline"]["scf"]
    assert scf["s_per_iter"] > 0 and len(scf["iteration_s"]) == 3 and scf["workers"] >= 1


def test_reference_arm_config_equals_ours():
    """Both arms print the same config object (the precision is a key of its own)."""
    import bench
    assert "precision" not in bench.WORKLOAD and bench.WORKLOAD["parallelism"] == "single GPU"


def test_reference_arm_loads_no_product_library():
    """The reference arm runs in a process that never maps liblres_gb300.so."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    code = ("import sys, types; sys.path.insert(0, %r); import bench\n"
            "from lresdft_gb300 import system\n"
            "cr = system.jittered_h2((2, 2, 2), a=4.5, bond=1.4, pts_per_cell=8, jitter=0.1, seed=0)\n"
            "bench.build_system = lambda cells=8, assembly='native': (cr, system.LCAOBasis(cr, assembly=assembly))\n"
            "bench.run_reference(types.SimpleNamespace(steps=1, warmup=3, scf_iters=0, cpu_scf=False))\n"
            "print('MAPPED', any('liblres_gb300' in l for l in open('/proc/self/maps')))\n") % root
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    assert "MAPPED False" in out.stdout


def test_clock_samples_parsed():
    """Only the samples inside the timed region count; with none inside, the nearest one."""
    import datetime
    import bench
    c = bench.Clocks()
    c.f.write("2026/12/04 10:00:00.050, 0, 1200, 2070, 400.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
              "2026/12/04 10:00:00.100, 0, 1965, 2070, 900.50, 0x0000000000000004, Not Active, Not Active, Not Active, Active\n"
              "2026/12/04 10:00:00.150, 0, 1980, 2070, 950.10, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
              "2026/12/04 10:00:00.200, 0, 2010, 2070, 990.00, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active\n"
              "2026/12/04 10:00:00.250, 0, 1100, 2070, 300.00, 0x0000000000000000, Active, Not Active, Not Active, Not Active\n")

    class Proc:
        def terminate(self):
            pass

        def wait(self):
            pass

    c.p = Proc()
    c.t0 = datetime.datetime(2026, 12, 4, 10, 0, 0, 90000)
    c.t1 = datetime.datetime(2026, 12, 4, 10, 0, 0, 210000)
    out = c.stop()
    assert out["sm_mhz"] == 1980.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["sw_power_cap"]
    t = datetime.datetime(2026, 12, 4, 10, 0, 0, 160000)
    lines = ["2026/12/04 10:00:00.100, 0, 1965, 2070, 900.50, 0x0, Not Active, Not Active, Not Active, Not Active",
             "2026/12/04 10:00:00.150, 0, 1980, 2070, 950.10, 0x0, Not Active, Not Active, Not Active, Not Active"]
    near = bench.Clocks.summarise(lines, t, t + datetime.timedelta(milliseconds=5))
    assert near["samples"] == 1 and near["sm_mhz"] == 1980.0


def test_algorithmic_flops():
    import bench
    nW = np.array([264, 288, 312])
    assert bench.algorithmic_flops(nW, 32) == 32 * (32.0 / 3.0) * float(np.sum(nW.astype(float) ** 3))


def test_reference_arm_other_ranks_do_nothing(monkeypatch, capsys):
    """Under torchrun only rank 0 runs the reference arm and prints its line."""
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr(bench, "build_system", lambda *a, **k: (_ for _ in ()).throw(AssertionError("ran")))
    bench.run_reference(types.SimpleNamespace(steps=1, warmup=3))
    assert capsys.readouterr().out == ""


def _rank_main(rank, world, port, out):
    import os
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")       # rank 1 is the slower one
    dist.barrier()
    out.put((rank, ms))
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks():
    """Under torchrun every timed leg of our arm reports the slowest rank's time: two gloo ranks
    on the CPU (spawned processes) both get the larger of their two times; without a process
    group the value is returned as it is."""
    import socket
    import torch.multiprocessing as mp
    import bench
    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(out.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert got == [(0, 15.0), (1, 15.0)]
    assert all(p.exitcode == 0 for p in procs)
