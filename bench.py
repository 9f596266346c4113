#!/usr/bin/env python
"""Benchmark of the sparse statevector gate path: amp-updates/s on one GB300.

Workload (default): the 40-qubit configuration -- a seeded 2000-gate circuit from |0...0>,
H on qubits 0..19 then 30% diagonal / 30% permutation / 40% branching gates with 0-3
controls, branching targets < 20 (at most 2^20 nonzeros), FP64 amplitudes, table load
factor 0.5. One step = the whole circuit from |0...0>. Synthetic data: the reference
publishes no benchmark circuits.

value   : sum over gates of input nonzeros / device time (CUDA events on the engine's
          stream, inputs resident, L2 flushed before every step).
e2e     : the same metric through the C ABI with host buffers: gate array host->device,
          state |0...0>, every gate, the final state read back to host arrays.
roofline: the gate-pass kernel; achieved = algorithmic bytes of the passes (device
          counter, see sqc_stats.alg_bytes) / their measured time; peak = the measured
          HBM copy bandwidth.
cpu_baseline / --impl reference: the CPU restatement of the reference algorithm
          (oracle/sparse_oracle.c, OpenMP over nonzeros) on a bounded prefix of the circuit.

Multi-GPU: independent replicas (one circuit per rank, different seeds), no collective on
the data path; value = all ranks' amp-updates / the slowest rank's time ("weak").
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

PROFILE_TXT = os.path.join(ROOT, "profiles", "pass_kernel_c2_fp64.txt")


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="sparqc", choices=["sparqc", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3"])
    ap.add_argument("--precision", type=int, default=64, choices=[64, 32])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="CPU baseline sample budget")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(name, rank):
    from sparqc_gb300 import circuits
    nq, g = circuits.config_circuit(name, index=rank, seed=0)
    p = circuits.CONFIGS[name]
    return nq, g, p


def config_dict(name, p, precision, world):
    return {"workload": f"{name}: {p['nq']} qubits, branching targets < {p['k']} (<= 2^{p['k']} nonzeros), "
                        f"{p['depth']} gates, 0-{p['max_controls']} controls, 30/30/40 diag/perm/branch, "
                        f"FP{precision}, load factor 0.5, seed 0",
            "qubits": p["nq"], "gates": p["depth"], "k": p["k"], "precision": f"fp{precision}",
            "l2": "flushed before every step (256 MiB write)", "parallelism": f"replicas x{world}"}


# --------------------------------------------------------------------------------------
# CPU baseline: the oracle's C restatement, timed on a bounded prefix of the circuit.
def cpu_run(gates, seconds, threads, precision):
    from oracle.sparse import SparseOracle
    o = SparseOracle(precision=precision, threads=threads)
    t0 = time.perf_counter()
    n = 0
    for i in range(gates.size):
        o.apply(gates[i:i + 1])
        n = i + 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    return o.amp_updates, dt, n


def cpu_baseline(gates, seconds, precision):
    from oracle.sparse import SparseOracle
    threads = max(1, SparseOracle.max_threads())
    upd, dt, n = cpu_run(gates, seconds, threads, precision)
    return {"value": upd / dt, "unit": "amp-updates/s", "cores": threads, "kind": "port",
            "sample": f"first {n} of {gates.size} gates ({upd:.3e} amp-updates in {dt:.1f} s), "
                      f"oracle/sparse_oracle.c, {threads} OpenMP threads"}


# --------------------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, device):
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{os.getpid()}.csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def read_profile_traffic():
    """Per-launch DRAM bytes of the gate-pass kernel from the committed ncu summary, if any."""
    try:
        for line in open(PROFILE_TXT):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":")[1])
    except OSError:
        pass
    return None


def measured_peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return None


# --------------------------------------------------------------------------------------
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    nq, gates, p = workload(args.workload, 0)
    from oracle.sparse import SparseOracle
    threads = max(1, SparseOracle.max_threads())
    per_step = max(2.0, min(20.0, 150.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_run(gates, per_step, threads, args.precision)
    tot_upd, tot_t, n = 0, 0.0, 0
    for _ in range(args.steps):
        upd, dt, n = cpu_run(gates, per_step, threads, args.precision)
        tot_upd += upd
        tot_t += dt
    v = tot_upd / tot_t
    sample = (f"each step: first {n} of {gates.size} gates of the workload ({per_step:.0f} s budget), "
              f"oracle/sparse_oracle.c (CPU restatement of the reference FC gate algorithm), {threads} OpenMP threads")
    out = {"metric": "amp-updates/s", "value": v, "unit": "amp-updates/s", "impl": "reference",
           "n_gpus": 0, "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": f"f{args.precision}",
           "data": "synthetic", "config": config_dict(args.workload, p, args.precision, 1),
           "cpu_baseline": {"value": v, "unit": "amp-updates/s", "cores": threads, "kind": "port", "sample": sample},
           "e2e": {"value": v, "unit": "amp-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from sparqc_gb300 import build as engine_build, engine
    engine_build.build()

    nq, gates, p = workload(args.workload, rank)
    stream = torch.cuda.current_stream()
    A = 16 if args.precision == 64 else 8
    st = engine.State(nq, precision=args.precision, stream=stream.cuda_stream,
                      initial_buckets=1 << max(6, p["k"] - 4 + 1))
    # warm-up: grows the tables to their final size and fixes the per-step counters
    for _ in range(max(3, args.warmup)):
        sw = st.stats()
        st.set_zero()
        st.apply(gates)
        st.sync()
    s0 = st.stats()
    upd_per_step = s0["amp_updates"]
    alg_per_step = s0["alg_bytes"]
    passes_per_step = s0["passes"] - sw["passes"]
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    launches0 = st.stats()["kernel_launches"]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(local) if rank == 0 else None
    t_wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(i & 0xFF)
        ev[i][0].record(stream)
        st.set_zero()
        st.apply(gates)
        st.flush()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall0
    clk = clocks.stop() if clocks else None
    if world > 1:
        torch.distributed.barrier()
    st.sync()
    s1 = st.stats()
    if s1["replays"] != s0["replays"]:
        raise RuntimeError("a timed step overflowed its table; warm-up did not size it")
    launches = s1["kernel_launches"] - launches0
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    t_dev = dev_ms / 1e3
    if world > 1:
        t = torch.tensor([t_dev], dtype=torch.float64, device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        t_max = float(t.item())
    else:
        t_max = t_dev
    value = upd_per_step * args.steps * world / t_max

    # e2e: through the C ABI with host buffers (gate array in, final state out)
    keys = np.empty(1 << p["k"], np.uint64)
    re = np.empty_like(keys, dtype=np.float64)
    im = np.empty_like(keys, dtype=np.float64)
    got = engine.ctypes.c_uint64()
    L = engine.load()
    gates_c = np.ascontiguousarray(gates)
    e2e_steps = max(3, min(args.steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    nout = 0
    for _ in range(e2e_steps):
        st.set_zero()
        st.apply(gates_c)
        rc = L.sqc_get_state(st.handle, keys.ctypes.data_as(engine.ctypes.c_void_p),
                             re.ctypes.data_as(engine.ctypes.c_void_p), im.ctypes.data_as(engine.ctypes.c_void_p),
                             keys.size, engine.ctypes.byref(got), 0)
        if rc != 0:
            raise RuntimeError(f"sqc_get_state failed: {rc}")
        nout = got.value
    e2e_t = (time.perf_counter() - t0) / e2e_steps
    e2e = {"value": upd_per_step * world / e2e_t, "unit": "amp-updates/s",
           "h2d_bytes_per_step": int(gates.size * 136), "d2h_bytes_per_step": int(nout * 24),
           "path": "sqc_set_zero_state + sqc_apply_gates (host gate array) + sqc_get_state (host arrays)"}

    if rank != 0:
        return
    peaks = measured_peaks()
    peak = peaks["hbm_gbs"] if peaks else 6800.0
    achieved = alg_per_step * args.steps / t_dev / 1e9
    traffic = read_profile_traffic()
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "traffic": traffic,
                "kernel": "pass_kernel (gate pass)", "algorithmic_bytes_per_step": alg_per_step,
                "peak_source": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks else "fallback 6.8 TB/s",
                "note": "achieved over the whole step (gate passes are all but one of its kernels)"}
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(gates, args.cpu_seconds, args.precision)
    out = {"metric": "amp-updates/s", "value": value, "unit": "amp-updates/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dev_ms / args.steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": f"f{args.precision}",
           "data": "synthetic", "config": config_dict(args.workload, p, args.precision, world),
           "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "gpu_launches": int(launches),
           "clocks": clk, "passes_per_step": passes_per_step, "gates_per_step": int(gates.size),
           "wall_s_timed": t_wall}
    print(json.dumps(out), flush=True)
    st.close()


def main():
    args = parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
