#!/usr/bin/env python
"""PC-stable skeleton benchmark on GB300: CI tests/s of the batched device engine.

One step = one full PC-stable skeleton (all levels, alpha 0.05) over the resident
synthetic dataset of the chosen configuration (default c2: 100 nodes, average
in-degree 2, cardinality U{2..5}, Dirichlet(0.5), 50,000 uint8 samples).
CI tests are the reference's deterministic sequential (group size 1) count.

  value      tests / device time (CUDA events on the engine's stream), dataset in HBM,
             L2 flushed (512 MB write) before every timed step
  e2e        same metric through the C ABI with host buffers: upload (H2D + relabel),
             skeleton, result fetch (D2H) inside the timed region
  plain      the same skeleton through the plain one-launch-per-test kernel
  roofline   counting+scoring kernel: algorithmic bytes (2+|Z|) * n_samples per test over
             its event-timed duration, against the measured HBM copy bandwidth
  cpu_baseline  the CPU oracle port (reference algorithm, int32 columns, OpenMP) on the host

--impl reference runs the CPU port as the reference arm (rank 0 only).
Multi-GPU (--gpus N under torchrun): independent replicas, one per rank ("replicas only").
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOADS = {
    "c1": "c1: 37 nodes, 46 edges, max in-degree 4, cardinality U{2,3,4}, Dirichlet(1), 5,000 uint8 samples",
    "c2": "c2: 100 nodes, avg in-degree 2 (max 5), cardinality U{2..5}, Dirichlet(0.5), 50,000 uint8 samples",
    "c3": "c3: 223 nodes, avg in-degree 1.5, cardinality 3, Dirichlet(1), 500,000 uint8 samples, |Z|<=4",
    "c4": "c4: 1,041 nodes, avg in-degree 1.3 (max 3), cardinality U{2..8} + 20% U{9..21}, Dirichlet(0.3), "
          "100,000 uint8 samples",
    "c5": "c5: 64 independent datasets in one engine, nodes U[20,200], samples log-uniform [1e3, 2e5], "
          "cardinality U{2..6}, avg in-degree U[1.5,2.5], Dirichlet(1)",
}
CPU_SAMPLE_JOBS = 8        # c5: the CPU arms time 8 datasets (a bounded sample) ...
CPU_SAMPLE_MAX_S = 40000   # ... the first 8 of at most 40,000 samples (one of 174,000 takes minutes)


def cpu_sample(data):
    """The datasets the CPU arms time, and what that sample is."""
    if len(data) == 1:
        return data, None
    pick = [r for r in data if r.shape[1] <= CPU_SAMPLE_MAX_S][:CPU_SAMPLE_JOBS]
    return pick, "the first %d of the %d datasets with at most %d samples" % (len(pick), len(data),
                                                                             CPU_SAMPLE_MAX_S)


def load_workload(name):
    """(list of raw uint8 [n, S] datasets, depth): one dataset, or c5's 64."""
    import fastpgm_gb300 as F
    if name == "c5":
        return F.make_jobs(F.c5_jobs())
    raw, depth, _ = F.make_config(name)
    return [raw], depth


def upload(eng, data):
    if len(data) == 1:
        eng.upload(data[0])
    else:
        eng.upload_jobs(data)



def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--alpha", type=float, default=0.05)
    ap.add_argument("--no-plain", action="store_true", help="skip the plain-kernel comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU-baseline run")
    ap.add_argument("--profile-one", action="store_true",
                    help="run exactly one skeleton (no warm-up, flush, e2e or baselines) for profilers; "
                         "prints its statistics, not a benchmark line")
    return ap.parse_args()


def run_profile_one(a):
    import fastpgm_gb300 as F
    data, depth = load_workload(a.config)
    with F.Engine(0) as eng:
        upload(eng, data)
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth).to_dict()
    print(json.dumps({"profile_one": a.config, "stats": st}))


class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch.distributed as dist
            backend = os.environ.get("FPGM_DIST_BACKEND", "gloo")
            dist.init_process_group(backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def allreduce(self, v, op):
        if not self.pg:
            return v
        import torch
        t = torch.tensor([float(v)], dtype=torch.float64)
        self.pg.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v):
        return self.allreduce(v, self.pg.ReduceOp.MAX) if self.pg else v

    def sum(self, v):
        return self.allreduce(v, self.pg.ReduceOp.SUM) if self.pg else v

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


class Clocks:
    """nvidia-smi sampling during the timed region (every 200 ms)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                      stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.flush()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                c = [x.strip() for x in line.split(",")]
                if len(c) >= 9:
                    rows.append(c)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        j = json.load(open(p))
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(kernels, config):
    """DRAM bytes of one captured launch (dram__bytes_read.sum + dram__bytes_write.sum), that
    launch's algorithmic bytes and the kernel captured, from the committed ncu summary of the
    first of `kernels` that has one for `config`; None when there is none."""
    for kernel in kernels:
        p = os.path.join(ROOT, "profiles", "%s_%s.txt" % (kernel, config))
        if os.path.exists(p):
            break
    else:
        return None
    got = {"kernel": kernel}
    for line in open(p):
        for key in ("dram_bytes_per_launch", "algorithmic_bytes_per_launch"):
            if line.startswith(key + ":"):
                got[key] = float(line.split(":")[1])
    return got.get("dram_bytes_per_launch"), got.get("algorithmic_bytes_per_launch"), got["kernel"]


def counting_phase(groups, peak):
    """The whole counting phase (every counting kernel group): summed algorithmic bytes over
    summed event time, against the HBM peak.  groups: [(kernel_ms, algorithmic_bytes)]."""
    ms = sum(g[0] for g in groups)
    nbytes = sum(g[1] for g in groups)
    if ms <= 0:
        return None
    ach = nbytes / (ms / 1e3) / 1e9
    return {"achieved": ach, "peak": peak, "unit": "GB/s", "frac": ach / peak, "kernel_ms": ms,
            "algorithmic_bytes": nbytes}


def cpu_port(data, depth, alpha, threads):
    """The oracle port over the datasets one after another: (tests, seconds)."""
    from oracle import oracle as O
    tests, dt = 0, 0.0
    for raw in data:
        cols, card = O.relabel(raw)
        t0 = time.perf_counter()
        r = O.pc_skeleton(cols, card, alpha=alpha, depth=depth, threads=threads)
        dt += time.perf_counter() - t0
        tests += sum(r["stats"]["tests"])
    return tests, dt


def run_reference(a, d):
    import fastpgm_gb300 as F
    if d.rank != 0:
        return
    data, depth = load_workload(a.config)
    sample, what = cpu_sample(data)
    what = (what + " per step") if what else "full %s skeleton per step" % a.config
    threads = os.cpu_count() or 1
    for _ in range(a.warmup):
        cpu_port(sample, depth, a.alpha, threads)
    tests, secs = 0, 0.0
    for _ in range(a.steps):
        t, s = cpu_port(sample, depth, a.alpha, threads)
        tests += t
        secs += s
    v = tests / secs
    line = {"impl": "reference", "metric": "CI tests/s (PC-stable skeleton, deterministic test count)", "value": v,
            "unit": "CI tests/s", "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": secs / a.steps * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u8 data, int32 counts, fp64 G2", "data": "synthetic (seeded random DAG + Dirichlet CPTs)",
            "config": {"workload": WORKLOADS[a.config], "alpha": a.alpha, "tests_per_step": tests // a.steps},
            "cpu_baseline": {"value": v, "unit": "CI tests/s", "cores": threads, "kind": "port",
                             "sample": what},
            "e2e": {"value": v, "unit": "CI tests/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def flush_l2(buf):
    import torch
    buf.zero_()
    torch.cuda.synchronize()


def run_ours(a, d):
    import torch
    import fastpgm_gb300 as F
    torch.cuda.set_device(d.local)
    data, depth = load_workload(a.config)
    eng = F.Engine(d.local)
    upload(eng, data)
    l2buf = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda:%d" % d.local)
    for _ in range(max(3, a.warmup)):
        eng.pc_skeleton(alpha=a.alpha, depth=depth)
    clocks = Clocks(d.local)
    clocks.start()
    d.barrier()
    torch.cuda.synchronize()
    tests = 0
    span_ms = 0.0
    count_ms = 0.0
    count_bytes = 0.0
    count_launches = 0
    large_ms = 0.0
    large_bytes = 0.0
    launches = 0
    last = None
    for _ in range(a.steps):
        flush_l2(l2buf)
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth).to_dict()
        tests += sum(st["tests"])
        span_ms += st["span_ms"]
        count_ms += st["count_ms"]
        count_bytes += st["count_bytes"]
        count_launches += st["count_launches"]
        large_ms += st["large_ms"]
        large_bytes += st["large_bytes"]
        launches += st["kernel_launches"]
        last = st
    torch.cuda.synchronize()
    d.barrier()
    clk = clocks.stop()
    t_max = d.max(span_ms / 1e3)
    tests_all = d.sum(tests)
    value = tests_all / t_max
    # end to end through the C ABI with host buffers: samples from pinned host memory
    # (upload + relabel), the skeleton, and the adjacency + sepset arrays back to the host
    pinned = [torch.from_numpy(raw).pin_memory().numpy() for raw in data]
    e2e_secs = 0.0
    e2e_tests = 0
    res = None
    for _ in range(a.steps):
        flush_l2(l2buf)
        t0 = time.perf_counter()
        upload(eng, pinned)
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth).to_dict()
        res = eng.result_arrays()
        e2e_secs += time.perf_counter() - t0
        e2e_tests += sum(st["tests"])
    e2e = d.sum(e2e_tests) / d.max(e2e_secs)
    n = sum(r.shape[0] for r in data)
    W = (n + 31) // 32
    d2h = n * W * 4 + len(res["removed"]) * 16 + len(res["sep_vars"]) * 4
    # plain one-launch-per-test kernel
    plain = None
    if not a.no_plain:
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth, mode=F.FPGM_MODE_PLAIN).to_dict()
        pt = sum(st["tests"])
        plain = {"value": pt / (st["span_ms"] / 1e3), "unit": "CI tests/s", "ms": st["span_ms"],
                 "kernel_launches": st["kernel_launches"]}
    peak, peak_kind = peaks()
    # the two counting kernels, timed with CUDA events on the engine's stream; the roofline
    # object describes the one with the larger share of device time
    kernels = []
    for name, desc, members, ms, nbytes in (
            ("ci_warp_kernel", "classify + warp-per-test + CTA-per-test kernels, shared-memory tables",
             ("ci_warp_kernel",), count_ms, count_bytes),
            ("ci_compact_kernel+ci_part_kernel",
             "tier 2, joint tables beyond shared memory: hashed strata (compact kernel) and, for tests of "
             "65,536+ samples whose strata overflow its shared hash, partitioned strata (partition kernel)",
             ("ci_part_kernel", "ci_compact_kernel"), large_ms, large_bytes)):
        if ms <= 0:
            continue
        ach = nbytes / (ms / 1e3) / 1e9
        tr = profiled_traffic(members, a.config)
        kernels.append({"kernel": name, "what": desc, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                        "frac": ach / peak, "peak_kind": peak_kind, "kernel_ms": ms, "algorithmic_bytes": nbytes,
                        "launches": count_launches if name == "ci_warp_kernel" else None,
                        "traffic": tr[0] if tr else None,
                        "traffic_launch_algorithmic_bytes": tr[1] if tr else None,
                        "traffic_kernel": tr[2] if tr else None})
    kernels.sort(key=lambda k: -k["kernel_ms"])
    roofline = dict(kernels[0])
    roofline["others"] = kernels[1:]
    roofline["counting_phase"] = counting_phase([(k["kernel_ms"], k["algorithmic_bytes"]) for k in kernels], peak)
    cpu = None
    if d.rank == 0 and d.world == 1 and not a.no_cpu:
        threads = os.cpu_count() or 1
        sample, what = cpu_sample(data)
        t, s = cpu_port(sample, depth, a.alpha, threads)
        what = what or "one full %s skeleton" % a.config
        cpu = {"value": t / s, "unit": "CI tests/s", "cores": threads, "kind": "port",
               "sample": "%s (%d tests, %.1f s)" % (what, t, s)}
    eng.close()
    if d.rank != 0:
        return
    line = {
        "metric": "CI tests/s (PC-stable skeleton, deterministic test count)", "value": value, "unit": "CI tests/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": max(3, a.warmup), "ms_per_step": t_max * 1e3 / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8 data, int32 counts, fp32 G2 (fp64 p-value and band recheck)",
        "data": "synthetic (seeded random DAG + Dirichlet CPTs, forward sampled)",
        "config": {"workload": WORKLOADS[a.config], "alpha": a.alpha, "tests_per_step": tests // a.steps,
                   "levels": last["n_levels"], "tests_per_level": last["tests"],
                   "tests_executed_per_level": last["tests_executed"], "edges_after": last["edges_after"],
                   "waves": last["waves"], "level_ms": [round(x, 3) for x in last["ms"]],
                   "large_table_ms": last["large_ms"], "l2": "flushed before each timed step (512 MB write)",
                   "parallelism": "replicas" if a.gpus > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "CI tests/s", "h2d_bytes_per_step": int(sum(r.nbytes for r in data)),
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "roofline": roofline,
        "plain": plain,
        "speedup_vs_plain": (value / plain["value"]) if plain else None,
        "precision": {"fp64_rechecks": last["rechecks"], "near_ties": last["near_ties"],
                      "max_abs_dp_fp32_vs_fp64": last["max_abs_dp"], "large_tests": last["large_tests"]},
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    print(json.dumps(line))


def main():
    a = parse()
    if a.profile_one:
        run_profile_one(a)
        return
    d = Dist()
    try:
        if a.impl == "reference":
            run_reference(a, d)
        else:
            run_ours(a, d)
    finally:
        d.close()


if __name__ == "__main__":
    main()
