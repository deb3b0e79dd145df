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


def load_workload(name, generate=None):
    """(list of raw uint8 [n, S] datasets, depth): one dataset, or c5's 64.  generate: the
    seeded sampler (default the engine library's; the CPU arms pass the oracle's copy so that
    they never load the engine)."""
    from fastpgm_gb300 import configs as C
    if name == "c5":
        return C.make_jobs(C.c5_jobs(), generate=generate)
    raw, depth, _ = C.make_config(name, generate=generate)
    return [raw], depth


def bench_config(a, depth):
    """The `config` object, identical in both arms."""
    return {"workload": WORKLOADS[a.config], "alpha": a.alpha, "depth": depth,
            "parallelism": "replicas" if a.gpus > 1 else "single GPU"}


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
    ap.add_argument("--no-north-star", action="store_true", help="skip the c4 (north-star workload) object")
    ap.add_argument("--no-wall", action="store_true", help="skip the BNSL_PCStable wall-time object")
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
    """The reference algorithm's CPU path (the oracle port, all host threads).  Loads only
    oracle/_build/*.so: the inputs come from the oracle's copy of the seeded sampler."""
    from oracle import oracle as O
    if d.rank != 0:
        return
    data, depth = load_workload(a.config, generate=O.generate)
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
            "dtype": "u8 data, int32 counts, fp64 G2", "data": "synthetic (seeded random DAG + Dirichlet CPTs, forward sampled)",
            "config": bench_config(a, depth), "tests_per_step": tests // a.steps,
            "cpu_baseline": {"value": v, "unit": "CI tests/s", "cores": threads, "kind": "port",
                             "sample": what},
            "e2e": {"value": v, "unit": "CI tests/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def flush_l2(buf):
    import torch
    buf.zero_()
    torch.cuda.synchronize()


def skeleton_run(eng, a, depth, steps, l2buf, clocks=None, d=None):
    """`steps` timed skeletons on a resident dataset, L2 flushed before each; the sums of the
    engine's per-call statistics (device span and the counting kernels' event times)."""
    import torch
    tot = {"tests": 0, "span_ms": 0.0, "count_ms": 0.0, "count_bytes": 0.0, "count_launches": 0, "large_ms": 0.0,
           "large_bytes": 0.0, "kernel_launches": 0, "gram_ms": 0.0, "gram_flops": 0.0, "gram_tests": 0}
    if clocks:
        clocks.start()
    if d:
        d.barrier()
    torch.cuda.synchronize()
    last = None
    for _ in range(steps):
        flush_l2(l2buf)
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth).to_dict()
        tot["tests"] += sum(st["tests"])
        for k in ("span_ms", "count_ms", "count_bytes", "count_launches", "large_ms", "large_bytes",
                  "kernel_launches", "gram_ms", "gram_flops", "gram_tests"):
            tot[k] += st[k]
        last = st
    torch.cuda.synchronize()
    if d:
        d.barrier()
    tot["clocks"] = clocks.stop() if clocks else None
    tot["last"] = last
    return tot


def e2e_run(eng, a, data, depth, steps, l2buf):
    """End to end through the C ABI: samples from pinned host memory (upload + relabel),
    the skeleton, the adjacency and separating sets back to the host.  (tests, seconds, d2h bytes)."""
    import torch
    pinned = [torch.from_numpy(raw).pin_memory().numpy() for raw in data]
    secs, tests, res = 0.0, 0, None
    for _ in range(steps):
        flush_l2(l2buf)
        t0 = time.perf_counter()
        upload(eng, pinned)
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth).to_dict()
        res = eng.result_arrays()
        secs += time.perf_counter() - t0
        tests += sum(st["tests"])
    n = sum(r.shape[0] for r in data)
    W = (n + 31) // 32
    d2h = n * W * 4 + len(res["removed"]) * 16 + len(res["sep_vars"]) * 4
    return tests, secs, d2h


def kernel_groups(tot, config, peak, peak_kind):
    """Roofline objects of the two counting-kernel groups (event-timed on the engine's stream),
    the larger share first."""
    kernels = []
    for name, desc, members, ms, nbytes in (
            ("ci_warp_kernel", "classify + warp-per-test + CTA-per-test kernels, shared-memory tables",
             ("ci_warp_kernel",), tot["count_ms"], tot["count_bytes"]),
            ("ci_compact_kernel+ci_part_kernel",
             "tier 2, joint tables beyond shared memory: hashed strata (compact kernel) and partitioned "
             "strata (partition kernels)", ("ci_part_kernel", "ci_compact_kernel"), tot["large_ms"],
             tot["large_bytes"])):
        if ms <= 0:
            continue
        ach = nbytes / (ms / 1e3) / 1e9
        tr = profiled_traffic(members, config)
        kernels.append({"kernel": name, "what": desc, "bound": "hbm", "achieved": ach, "peak": peak, "unit": "GB/s",
                        "frac": ach / peak, "peak_kind": peak_kind, "kernel_ms": ms, "algorithmic_bytes": nbytes,
                        "launches": tot["count_launches"] if name == "ci_warp_kernel" else None,
                        "traffic": tr[0] if tr else None,
                        "traffic_source": ("profiles/%s_%s.txt (one ncu capture; not measured in this run)"
                                           % (tr[2], config)) if tr else None,
                        "traffic_launch_algorithmic_bytes": tr[1] if tr else None})
    kernels.sort(key=lambda k: -k["kernel_ms"])
    return kernels


def tensor_peak():
    """Dense FP8 tensor rate: twice the measured bf16 GEMM burst (FP8 runs at twice the bf16
    rate on this part; no FP8 figure is measured), else twice the fallback."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return 2.0 * float(json.load(open(p))["bf16_tflops"]), "fp8 dense = 2 x measured bf16 burst"
    return 2.0 * 1900.0, "fp8 dense = 2 x fallback bf16 burst"


def gram_roofline(tot):
    """Level 0 on the tensor cores: Gram GEMM flops over the event time of the whole level-0
    wave (one-hot build + GEMM + pair scoring), against the dense FP8 tensor rate."""
    if tot["gram_ms"] <= 0:
        return None
    peak, kind = tensor_peak()
    ach = tot["gram_flops"] / (tot["gram_ms"] / 1e3) / 1e12
    return {"kernel": "gram_kernel", "what": "level 0: E4M3 one-hot Gram GEMM on tcgen05 (TMA-staged, FP32 in TMEM) + "
                                            "one-hot build + pair scoring", "bound": "tensor", "achieved": ach,
            "peak": peak, "unit": "TFLOP/s", "frac": ach / peak, "peak_kind": kind, "kernel_ms": tot["gram_ms"],
            "flops": tot["gram_flops"], "tests": tot["gram_tests"]}


def level_record(st):
    return {"levels": st["n_levels"], "tests_per_level": st["tests"], "tests_executed_per_level": st["tests_executed"],
            "edges_after": st["edges_after"], "waves": st["waves"], "level_ms": [round(x, 3) for x in st["ms"]],
            "large_table_ms": st["large_ms"], "graph_build_ms": round(st["graph_ms"], 3)}


def recorded(name):
    """A measurement kept under profiles/ as 'key: value' lines (see the file for its command)."""
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    out = {}
    for line in open(p):
        if ":" in line and not line.startswith((" ", "#", "|")):
            k, v = line.split(":", 1)
            out[k.strip()] = v.strip()
    return out


def north_star_c4(a, l2buf, peak, peak_kind):
    """The spec workload (c4: 1,041 nodes, 100,000 samples) on the same engine build:
    device and end-to-end CI tests/s, the counting phase against the HBM roofline, and the
    plain one-launch-per-test kernel's rate from its recorded full run."""
    import fastpgm_gb300 as F
    sub = argparse.Namespace(**vars(a))
    sub.config = "c4"
    data, depth = load_workload("c4")
    with F.Engine(0) as eng:
        upload(eng, data)
        eng.pc_skeleton(alpha=a.alpha, depth=depth)
        tot = skeleton_run(eng, sub, depth, 2, l2buf, clocks=Clocks(0))
        tests, secs, d2h = e2e_run(eng, sub, data, depth, 1, l2buf)
    value = tot["tests"] / (tot["span_ms"] / 1e3)
    kernels = kernel_groups(tot, "c4", peak, peak_kind)
    plain = recorded("plain_kernel_c4.md")
    out = {"workload": WORKLOADS["c4"], "steps": 2, "value": value, "unit": "CI tests/s",
           "ms_per_step": tot["span_ms"] / 2, "tests_per_step": tot["tests"] // 2,
           "e2e": {"value": tests / secs, "unit": "CI tests/s", "h2d_bytes_per_step": int(sum(r.nbytes for r in data)),
                   "d2h_bytes_per_step": d2h},
           "counting_phase": counting_phase([(k["kernel_ms"], k["algorithmic_bytes"]) for k in kernels], peak),
           "kernel_groups": [{k: g[k] for k in ("kernel", "frac", "kernel_ms", "algorithmic_bytes")} for g in kernels],
           "tensor": gram_roofline(tot),
           "gpu_launches_per_step": tot["kernel_launches"] // 2, "clocks": tot["clocks"]}
    out.update(level_record(tot["last"]))
    if plain and "value" in plain:
        pv = float(plain["value"])
        out["plain"] = {"value": pv, "unit": "CI tests/s", "measured": plain.get("date"),
                        "source": "profiles/plain_kernel_c4.md (full plain skeleton, recorded run; too long to "
                                  "repeat in every bench run)"}
        out["speedup_vs_plain"] = value / pv
    return out


def wall_bnsl(configs, verbose=1):
    """Full BNSL_PCStable seconds through the C ABI (fpgm_bnsl_pcstable): CSV load, skeleton,
    orientation and the _struct file, the reference's whole learning job (fastpgm_api.cpp:18-44).
    The CSV is written beforehand (untimed); one untimed call first so the shared engine exists.
    The job's own report ("pc-stable step 1" = skeleton, "pc-stable" = skeleton + orientation)
    is read from its standard output."""
    import ctypes
    import fastpgm_gb300 as F
    libc = ctypes.CDLL(None)
    out = {}
    tmp = tempfile.mkdtemp(prefix="fpgm_wall_")
    try:
        for name in configs:
            data, depth = load_workload(name)
            csv = os.path.join(tmp, name + ".csv")
            F.write_csv(csv, data[0])
            rec = None
            for rep in range(2):
                log = os.path.join(tmp, "stdout.txt")
                sys.stdout.flush()
                saved = os.dup(1)
                fd = os.open(log, os.O_WRONLY | os.O_CREAT | os.O_TRUNC)
                os.dup2(fd, 1)
                try:
                    t0 = time.perf_counter()
                    F.bnsl_pcstable(verbose, os.cpu_count() or 1, 1, 0.05, "", csv, True)
                    secs = time.perf_counter() - t0
                finally:
                    libc.fflush(None)  # the job writes through C stdio: flush before fd 1 goes back
                    os.dup2(saved, 1)
                    os.close(saved)
                    os.close(fd)
                text = open(log).read()
                step1 = [l for l in text.splitlines() if l.startswith("pc-stable step 1:")]
                full = [l for l in text.splitlines() if l.startswith("pc-stable:")]
                rec = {"seconds": secs, "csv_mb": os.path.getsize(csv) / 1e6,
                       "skeleton_s": float(step1[-1].split(":")[1].split()[0]) if step1 else None,
                       "pc_stable_s": float(full[-1].split(":")[1].split()[0]) if full else None}
            if rec["pc_stable_s"] is not None:
                rec["orientation_s"] = rec["pc_stable_s"] - (rec["skeleton_s"] or 0.0)
                rec["load_and_write_s"] = rec["seconds"] - rec["pc_stable_s"]
            out[name] = rec
    finally:
        import shutil
        shutil.rmtree(tmp, ignore_errors=True)
    return out


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
    tot = skeleton_run(eng, a, depth, a.steps, l2buf, clocks=Clocks(d.local), d=d)
    t_max = d.max(tot["span_ms"] / 1e3)
    tests_all = d.sum(tot["tests"])
    value = tests_all / t_max
    e2e_tests, e2e_secs, d2h = e2e_run(eng, a, data, depth, a.steps, l2buf)
    e2e = d.sum(e2e_tests) / d.max(e2e_secs)
    # plain one-launch-per-test kernel
    plain = None
    if not a.no_plain:
        st = eng.pc_skeleton(alpha=a.alpha, depth=depth, mode=F.FPGM_MODE_PLAIN).to_dict()
        pt = sum(st["tests"])
        plain = {"value": pt / (st["span_ms"] / 1e3), "unit": "CI tests/s", "ms": st["span_ms"],
                 "kernel_launches": st["kernel_launches"]}
    peak, peak_kind = peaks()
    kernels = kernel_groups(tot, a.config, peak, peak_kind)
    roofline = dict(kernels[0]) if kernels else {"kernel": None}
    roofline["others"] = kernels[1:]
    roofline["counting_phase"] = counting_phase([(k["kernel_ms"], k["algorithmic_bytes"]) for k in kernels], peak)
    roofline["tensor"] = gram_roofline(tot)
    cpu, sample_gpu = None, None
    if d.rank == 0 and d.world == 1 and not a.no_cpu:
        threads = os.cpu_count() or 1
        sample, what = cpu_sample(data)
        t, s = cpu_port(sample, depth, a.alpha, threads)
        what = what or "one full %s skeleton" % a.config
        cpu = {"value": t / s, "unit": "CI tests/s", "cores": threads, "kind": "port",
               "sample": "%s (%d tests, %.1f s)" % (what, t, s)}
        if len(sample) < len(data):  # the GPU on the very datasets the CPU timed
            with F.Engine(d.local) as e2:
                upload(e2, sample)
                e2.pc_skeleton(alpha=a.alpha, depth=depth)
                ts = skeleton_run(e2, a, depth, 2, l2buf)
            sample_gpu = {"value": ts["tests"] / (ts["span_ms"] / 1e3), "unit": "CI tests/s",
                          "tests_per_step": ts["tests"] // 2, "sample": what}
    eng.close()
    ns, wall = None, None
    if d.rank == 0 and d.world == 1 and not a.no_north_star and a.config != "c4":
        ns = north_star_c4(a, l2buf, peak, peak_kind)
    if d.rank == 0 and d.world == 1 and not a.no_wall:
        wall = wall_bnsl(["c2", "c4"])
    if d.rank != 0:
        return
    line = {
        "metric": "CI tests/s (PC-stable skeleton, deterministic test count)", "value": value, "unit": "CI tests/s",
        "n_gpus": a.gpus, "steps": a.steps, "warmup": max(3, a.warmup), "ms_per_step": t_max * 1e3 / a.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "u8 data, int32 counts, fp32 G2 (fp64 p-value and band recheck)",
        "data": "synthetic (seeded random DAG + Dirichlet CPTs, forward sampled)",
        "config": bench_config(a, depth),
        "tests_per_step": tot["tests"] // a.steps,
        "l2": "flushed before each timed step (512 MB write)",
        "levels": level_record(tot["last"]),
        "e2e": {"value": e2e, "unit": "CI tests/s", "h2d_bytes_per_step": int(sum(r.nbytes for r in data)),
                "d2h_bytes_per_step": d2h},
        "gpu_launches": tot["kernel_launches"],
        "roofline": roofline,
        "plain": plain,
        "speedup_vs_plain": (value / plain["value"]) if plain else None,
        "precision": {"fp64_rechecks": tot["last"]["rechecks"], "near_ties": tot["last"]["near_ties"],
                      "max_abs_dp_fp32_vs_fp64": tot["last"]["max_abs_dp"],
                      "large_tests": tot["last"]["large_tests"]},
        "autotuner": {"what": "online: per (samples, |Z|, cells/samples) bucket the tier-2 tests are timed with "
                              "both methods (partition kernel, global strata hash); the faster is preferred",
                      "buckets_timed_both_ways": tot["last"]["tune_buckets"],
                      "buckets_preferring_partitions": tot["last"]["tune_partition"],
                      "tests_timed": tot["last"]["tune_timed"]},
        "cpu_baseline": cpu,
        "gpu_on_cpu_sample": sample_gpu,
        "north_star": ns,
        "wall": wall,
        "clocks": tot["clocks"],
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
