#!/usr/bin/env python
"""Throughput benchmark of the per-timestep MHD update on GB300.

Workload (the metric's configuration): 256^3 periodic decaying MHD turbulence
(seeded Gaussian-random solenoidal v and B, E(k) ~ k^-2 on 2 <= k <= 8, rms 1.0
and 0.5, rho = 1, Ms = 0.5), PDM reconstruction + RK2, FP32 state and fluxes
with FP64 metric and sums.  One step = one full RK2 step of the whole grid.

Prints ONE JSON line (rank 0).  ``value`` = zone-updates/s over K device-timed
steps (CUDA events on the solver's stream, graph replay, inputs resident);
``e2e`` = the same metric through the C ABI with host FP64 buffers: mhd_init
(H2D), K x mhd_step with tau/status read back, mhd_fetch of the output fields
(D2H), all inside the timed region.

``--impl reference`` times the reference algorithm on the host cores instead
(the oracle port in its array-pass mode: no Fortran compiler exists to build
the reference itself), one RK2 step of the same 256^3 workload per timed step,
at most 20 timed steps.

The line also carries ``fp64`` (the same workload in all-FP64 mode) and
``equal_time`` (relative L1 error against the FP64 256^3 solve of FP32 and
FP64 runs at comparable GPU time), both measured after the timed region.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# Algorithmic (compulsory) HBM words per zone and stage of each launch family
# (FP32 = 4 B per word), averaged over the two RK2 stages:
#   flux_x: read 8 cell fields, write 8 x-face fluxes                     16
#   flux_y: read 8 cell fields + 8 x-face fluxes, write 8 divergences     24
#   flux_z_update: read 8 cell fields + 8 divergences + U^n (5, stage 2
#           only: 2.5 on average), write 5 primitives                     23.5
#   emf: per edge family read v1, v2, b1, b2, vf, write E (3 launches)   18
#   ct (CT fused with get_bxyz and vf, then the ghost shell): read 3 face B +
#           3 EMFs (+3 B^n on stage 2: 1.5) + the new rho, v (4), write 3 face
#           B + cell B and vf (4)                                            18.5
WORDS = {"flux_x": 16, "flux_y": 24, "flux_z_update": 23.5, "emf": 18, "ct": 18.5}
LAUNCHES = {"flux_x": 1, "flux_y": 1, "flux_z_update": 1, "emf": 3, "ct": 1}
RECON_NAMES = {1: "PDM", 2: "TVD", 3: "WENO5", 4: "MPWENO5", 5: "TVD-MC"}
# the sources of the step kernels: counts and traffic read from profiles/
# describe the code only while this hash matches the one stored beside them
STEP_SOURCES = ("mhd_kernels.cuh", "mhd_state.h", "mhd_api.cu", "mhd_fp32.cu")


def step_sources_sha16() -> str:
    h = hashlib.sha256()
    for name in STEP_SOURCES:
        h.update((ROOT / "mhd3d_mpi_fortran_gb300" / "csrc" / name).read_bytes())
    return h.hexdigest()[:16]


def profile_file(name: str):
    """(data, provenance) of a machine-readable profile summary; provenance
    says whether it was captured on the current step kernels."""
    f = ROOT / "profiles" / name
    if not f.exists():
        return None, None
    d = json.loads(f.read_text())
    sha = d.get("kernels_sha16") if isinstance(d, dict) else None
    return d, {"file": f"profiles/{name}", "kernels_sha16": sha, "stale": sha != step_sources_sha16()}


# kernel name -> launch family of the step (counts and traffic summaries)
def _family(kernel: str) -> str | None:
    k = kernel.split("(")[0]
    if "k_cfl" in k:
        return "dt"
    if "k_emf_pdm" in k or "k_emf_weno" in k or "k_emf<" in k or "k_emf_stream" in k or "k_emf_rows" in k:
        return "emf"
    if "k_flux_sweep" in k or "k_flux_t" in k:
        return "flux_y" if ", 1," in k.split("<", 1)[1][:12] else "flux_z_update"
    if "k_flux<" in k:
        return "flux_x"
    if "k_ct_fill" in k or "k_fill_bxyz" in k or "k_update_b" in k:
        return "ct"
    return None


def _ncu_rows(csv_path: str):
    """(kernel name, {metric: value}) per launch of an ncu --csv log, in order."""
    import csv
    rows = list(csv.reader(open(csv_path)))
    hi = next(i for i, r in enumerate(rows) if r and r[0] == "ID")
    h = rows[hi]
    ix = {k: i for i, k in enumerate(h)}
    out, cur = [], None
    for r in rows[hi + 1:]:
        if len(r) < len(h):
            continue
        key = (r[ix["ID"]], r[ix["Kernel Name"]])
        if cur is None or cur[0] != key:
            cur = (key, {})
            out.append(cur)
        v = r[ix["Metric Value"]].replace(",", "")
        try:
            cur[1][r[ix["Metric Name"]]] = float(v)
        except ValueError:
            pass
    return [(k[1], m) for k, m in out]


# launches per RK2 step of each kernel class, for per-step sums of captures
# that hold only some of a class's launches
_PER_STEP = {"dt": 1, "emf": 6, "emf_rows": 2, "flux_x": 2, "flux_y": 2, "flux_z_update": 2, "ct_fill": 2,
             "shell": 2}


def _class(kernel: str) -> str | None:
    f = _family(kernel)
    if f == "ct":
        return "shell" if "k_fill_bxyz" in kernel else "ct_fill"
    if f == "emf" and "k_emf_rows" in kernel:
        return "emf_rows"
    return f


def _step_sums(paths, metric_fn) -> dict:
    """Per-step sums of metric_fn(metrics) per launch family over ncu captures
    (comma-separated csv paths, one kernel each, a few launches), each class
    scaled from its captured launches to its launches per RK2 step."""
    acc, cnt = {}, {}
    for path in paths.split(","):
        for name, m in _ncu_rows(path):
            c = _class(name)
            if c is None:
                continue
            v = metric_fn(m)
            for key, val in v.items():
                acc.setdefault(c, {}).setdefault(key, 0.0)
                acc[c][key] += val
            cnt[c] = cnt.get(c, 0) + 1
    fam = {}
    for c, vals in acc.items():
        f = "ct" if c in ("ct_fill", "shell") else "emf" if c == "emf_rows" else c
        e = fam.setdefault(f, {})
        for key, val in vals.items():
            e[key] = e.get(key, 0.0) + val * _PER_STEP[c] / cnt[c]
    return fam


def _counts_of(m) -> dict:
    flop = (m.get("smsp__sass_thread_inst_executed_op_fadd_pred_on.sum", 0)
            + m.get("smsp__sass_thread_inst_executed_op_fmul_pred_on.sum", 0)
            + 2 * m.get("smsp__sass_thread_inst_executed_op_ffma_pred_on.sum", 0)
            + 2 * m.get("smsp__sass_thread_inst_executed_op_fadd2_pred_on.sum", 0)
            + 2 * m.get("smsp__sass_thread_inst_executed_op_fmul2_pred_on.sum", 0)
            + 4 * m.get("smsp__sass_thread_inst_executed_op_ffma2_pred_on.sum", 0))
    return {"flop": flop, "inst": m.get("smsp__thread_inst_executed.sum", 0),
            "us_ncu": m.get("gpu__time_duration.sum", 0) / 1e3,
            "dram_bytes": m.get("dram__bytes_read.sum", 0) + m.get("dram__bytes_write.sum", 0)}


def ingest_counts(a):
    """profiles/counts_pdm_rk2_fp32.json and profiles/traffic.json from ncu
    captures of `bench.py --n N --tiles T,E --profile-only`, one kernel per
    capture (--ingest-counts a.csv,b.csv,...): FP32 flop and thread
    instructions per zone-update of one RK2 step, per family and in total, and
    DRAM bytes per launch; stamped with the hash of the step sources they were
    captured on.  Traffic is scaled from the N^3 capture to a 256^3 launch by
    the units processed (x (256/N)^3)."""
    fam = _step_sums(a.ingest_counts, _counts_of)
    n3 = float(a.n) ** 3
    tot = {"flop": sum(e["flop"] for e in fam.values()) / n3, "inst": sum(e["inst"] for e in fam.values()) / n3}
    td, ey = (int(t) for t in a.tiles.split(","))
    key = f"td{td}_ei{ey}"
    p = ROOT / "profiles" / "counts_pdm_rk2_fp32.json"
    d = json.loads(p.read_text()) if p.exists() else {}
    if d.get("kernels_sha16") != step_sources_sha16():
        d = {}  # counts of older kernels do not mix with these
    d["kernels_sha16"] = step_sources_sha16()
    d["source"] = (f"ncu --metrics smsp__thread_inst_executed.sum, sm__sass_thread_inst_executed_op_"
                   f"{{fadd,fmul,ffma,fadd2,fmul2,ffma2}}_pred_on.sum, dram__bytes_{{read,write}}.sum, one kernel "
                   f"per capture (-k, <= 4 launches) of bench.py --n {a.n} --tiles T,E --steps 2 --warmup 3 "
                   f"--profile-only, scaled to one RK2 step, per zone-update of the {a.n}^3 grid; T = 32 is the "
                   f"column-sweep face shape")
    d["units"] = {"flop": "FP32 flop (fadd + fmul + 2 ffma + 2 fadd2 + 2 fmul2 + 4 ffma2 thread instructions)",
                  "inst": "thread instructions executed"}
    d.setdefault("per_zone_update", {})[key] = {k: round(v, 1) for k, v in tot.items()}
    d.setdefault("per_family_per_step", {})[key] = {
        f: {"flop": round(e["flop"] / n3, 1), "inst": round(e["inst"] / n3, 1), "us_ncu": round(e["us_ncu"], 1)}
        for f, e in fam.items()}
    p.write_text(json.dumps(d, indent=1) + "\n")
    scale = (256.0 / a.n) ** 3
    launches = {"emf": 6, "flux_x": 2, "flux_y": 2, "flux_z_update": 2, "ct": 2, "dt": 1}
    t = {"kernels_sha16": step_sources_sha16(),
         "source": f"dram__bytes_read.sum + dram__bytes_write.sum of the same captures at {a.n}^3, per launch of "
                   f"each family (CT + bxyz and its ghost shell counted as one, an EMF family with its share of the "
                   f"boundary-row launch), scaled x{scale:g} to a 256^3 launch "
                   f"(traffic grows with the units processed: every array of these kernels exceeds L2 at 256^3)",
         "captured_at": a.n,
         "per_launch": {f: e["dram_bytes"] * scale / launches[f] for f, e in fam.items()},
         "per_step_bytes_256": sum(e["dram_bytes"] for e in fam.values()) * scale}
    (ROOT / "profiles" / "traffic.json").write_text(json.dumps(t, indent=1) + "\n")
    print(json.dumps({"per_zone_update": d["per_zone_update"][key], "traffic": t["per_launch"]}))


def bench_config(n: int, recon: int) -> dict:
    """The workload both arms run (same keys and values in both lines)."""
    return {"workload": f"{n}^3 periodic decaying MHD turbulence (seeded solenoidal v and B, k^-2 on "
                        f"2<=k<=8), {RECON_NAMES[recon]} + RK2", "grid": [n, n, n], "recon": recon,
            "stepper": "RK2", "l2": "inputs larger than L2 (state >= 0.9 GB), no flush"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--recon", type=int, default=1)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--profile-only", action="store_true", help="short run for ncu (no JSON extras)")
    ap.add_argument("--tiles", default=None,
                    help="launch shapes 'face_tile,ei_tile' (e.g. 8,8) instead of the autotuner's choice")
    ap.add_argument("--ensemble", type=int, default=0,
                    help="batched-ensemble mode: this many periodic OT grids of sizes {32,48,64,96}^3")
    ap.add_argument("--no-study", action="store_true",
                    help="skip the FP64 line and the error-at-equal-GPU-time table")
    ap.add_argument("--study-steps", type=int, default=20)
    ap.add_argument("--ingest-counts", default=None,
                    help="write profiles/counts_pdm_rk2_fp32.json and traffic.json from these ncu csvs (ingest_counts)")
    ap.add_argument("--ensemble-key", type=int, default=256,
                    help="grids of the batched ensemble measured after the timed region (0: skip)")
    return ap.parse_args()


def roofs(zu_per_gpu: float, clocks: dict, recon: int, tiles) -> dict:
    """FP32 and instruction-issue rooflines of the whole step from per
    zone-update counts that ncu measured on the same kernels (FP32 flops =
    fadd + fmul + 2 ffma thread instructions; thread instructions issued),
    profiles/counts_pdm_rk2_fp32.json.  Peaks: SMs x 128 FP32 lanes x 2 flop
    and SMs x 4 schedulers x 32 lanes per cycle, at the median SM clock seen
    during the timed region."""
    counts, prov = profile_file("counts_pdm_rk2_fp32.json")
    if recon != 1 or counts is None:
        return {}
    key = f"td{tiles[0]}_ei{tiles[1]}"
    if key not in counts["per_zone_update"]:
        return {}
    c = counts["per_zone_update"][key]
    from mhd3d_mpi_fortran_gb300 import abi
    import ctypes as C
    info = (C.c_int32 * 4)()
    if abi.load().mhd_device_info(info) != 0:
        return {}
    sms, mhz = info[0], clocks.get("sm_mhz") or info[3]
    fp32_peak = sms * 128 * 2 * mhz * 1e6
    issue_peak = sms * 4 * 32 * mhz * 1e6
    return {
        "fp32_roof": {"flop_per_zone_update": c["flop"], "achieved_tflops": zu_per_gpu * c["flop"] / 1e12,
                      "peak_tflops": fp32_peak / 1e12, "frac": zu_per_gpu * c["flop"] / fp32_peak,
                      "peak_kind": f"nominal: {sms} SMs x 128 lanes x 2 flop x {mhz:.0f} MHz"},
        "issue_roof": {"inst_per_zone_update": c["inst"], "achieved_tinst_s": zu_per_gpu * c["inst"] / 1e12,
                       "peak_tinst_s": issue_peak / 1e12, "frac": zu_per_gpu * c["inst"] / issue_peak,
                       "peak_kind": f"nominal: {sms} SMs x 4 x 32 thread instructions x {mhz:.0f} MHz",
                       "counts_from": counts["source"]},
        "counts_provenance": prov,
    }


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.p.kill()

    def summary(self):
        if not self.p:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = [r.split(",") for r in Path(self.f.name).read_text().strip().splitlines() if r.strip()]
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for nm, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def workload(n):
    from mhd3d_mpi_fortran_gb300 import ics
    s = ics.turbulence(n, seed=0)
    # fixed RK dt below the initial CFL dt: the flow speeds up as it decays,
    # and the step must stay under the CFL limit for the whole run
    return s, 0.8 * ics.cfl_dt(s, cfl=0.3)


_CPU_STATES = {}


def cpu_rate(n, steps, recon=1, fused=False):
    """Oracle (FP64 restatement of the reference) zone-updates/s on the host:
    the reference's array passes, or with fused=True one pass per face / edge
    family (the same results)."""
    from mhd3d_mpi_fortran_gb300 import ics
    from mhd3d_mpi_fortran_gb300.abi import Params
    from oracle.oracle import OracleSolver, threads
    if n not in _CPU_STATES:
        _CPU_STATES[n] = ics.turbulence(n, seed=0)
    s = _CPU_STATES[n]
    prm = Params(n, n, n, reconop=recon, stepop=2, tau=ics.cfl_dt(s, cfl=0.3))
    o = OracleSolver(prm, s)
    o.set_fused(fused)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return n ** 3 * steps / dt, dt, threads()


def cpu_detail(recon=1):
    """The oracle in both modes (the reference's array passes; fused) on all
    host threads and on one, at 64^3 (2 RK2 steps each) and at 256^3 on all
    threads (1 step): the rates the reference's own CPU path would be
    compared at."""
    from oracle.oracle import threads, set_threads
    allt = threads()
    rows = []
    for mode, n, steps, t in [(m, n, st, t) for m in ("array", "fused")
                              for n, st, t in ((64, 2, allt), (64, 2, 1), (256, 1, allt))]:
        set_threads(t)
        v, dt, cores = cpu_rate(n, steps, recon, fused=(mode == "fused"))
        rows.append({"mode": mode, "grid": n, "steps": steps, "cores": cores, "value": v, "unit": "zone-updates/s",
                     "seconds": dt})
    set_threads(allt)
    _CPU_STATES.clear()
    return rows


REF_MAX_TIMED_STEPS = 20  # 256^3 array-pass steps take ~4.6 s on 16 Grace cores


def run_reference(a):
    """The reference's CPU path on the host cores: the FP64 oracle restatement
    in its array-pass mode (the reference's own per-routine passes and
    temporaries), all host threads, on the same workload as our arm (same
    config); each step is one RK2 step of the whole grid.  At most
    REF_MAX_TIMED_STEPS steps are timed so that the run stays within minutes;
    the line's `steps` says how many."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    n = a.n
    from mhd3d_mpi_fortran_gb300 import ics
    from mhd3d_mpi_fortran_gb300.abi import Params
    from oracle.oracle import OracleSolver, threads
    s, tau = workload(n)
    prm = Params(n, n, n, reconop=a.recon, stepop=2, tau=tau)
    o = OracleSolver(prm, s)
    o.step(max(1, min(a.warmup, 1)))
    k = max(1, min(a.steps, REF_MAX_TIMED_STEPS))
    t0 = time.perf_counter()
    o.step(k)
    dt = time.perf_counter() - t0
    o.close()
    v = n ** 3 * k / dt
    line = {
        "impl": "reference", "metric": "zone-updates/s", "value": v, "unit": "zone-updates/s",
        "n_gpus": a.gpus, "steps": k, "warmup": max(1, min(a.warmup, 1)), "ms_per_step": 1e3 * dt / k,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic: seeded solenoidal turbulence (same generator and seed as our arm)",
        "config": bench_config(n, a.recon),
        "cpu_baseline": {"value": v, "unit": "zone-updates/s", "cores": threads(), "kind": "port",
                         "sample": f"{k} RK2 steps of the {n}^3 workload (requested {a.steps}), FP64 oracle "
                                   f"restatement in array-pass mode, as the reference computes"},
        "e2e": {"value": v, "unit": "zone-updates/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def job_time_ms(ms_local: float, pg) -> float:
    """The job's time for the timed steps: the slowest rank's (max over ranks;
    every rank passed a barrier right before its timed region)."""
    if pg is None:
        return ms_local
    import torch
    t = torch.tensor([ms_local], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(n: int, steps: int, ws: int, ms: float) -> float:
    """Zone-updates/s of the whole job: every rank advances its own n^3 replica."""
    return n ** 3 * steps * ws / (ms * 1e-3)


def e2e_run(prm, s, n: int, ke: int) -> dict:
    """The metric end to end through the C ABI with host FP64 buffers:
    mhd_init (allocation, H2D of the FP64 state, ghost fill), ke x mhd_step
    (one RK2 step each, tau and status read back) and mhd_fetch (D2H of the
    11 FP64 output arrays into the caller's existing arrays), host wall clock."""
    from mhd3d_mpi_fortran_gb300 import MHDSolver
    from mhd3d_mpi_fortran_gb300.solver import output_arrays
    # the caller's FP64 arrays exist and hold data before the run, as the
    # Fortran driver's module arrays do after `initialization`
    dst = output_arrays(prm)
    for v in dst.values():
        v.fill(1.0)
    t0 = time.perf_counter()
    sv = MHDSolver(prm, s)
    t1 = time.perf_counter()
    for _ in range(ke):
        sv.step(1)
    t2 = time.perf_counter()
    sv.fetch(out=dst)
    t3 = time.perf_counter()
    el = t3 - t0
    sv.close()  # teardown (frees the device buffers) is not part of the run
    # FP64 host arrays copied as they are (the library converts on the device):
    # 5 cell + 3 face arrays in, 8 cell + 3 face arrays out, + tau/status per step
    nx, ny, nz = prm.shape
    cell, faces = nx * ny * nz, (nx + 1) * ny * nz + nx * (ny + 1) * nz + nx * ny * (nz + 1)
    h2d = 8 * (5 * cell + faces)
    d2h = 8 * (8 * cell + faces) + ke * 48
    return {"value": n ** 3 * ke / el, "unit": "zone-updates/s", "h2d_bytes_per_step": int(h2d / ke),
            "d2h_bytes_per_step": int(d2h / ke), "steps": ke, "seconds": el,
            "split_s": {"init": t1 - t0, "steps": t2 - t1, "fetch": t3 - t2},
            "how": "new handle in a warm process (the kernels are loaded), measured before the timed region"}


def run_ours(a):
    ws, rank, local = dist_env()
    if ws > 1:
        os.environ["CUDA_VISIBLE_DEVICES"] = str(local)
    from mhd3d_mpi_fortran_gb300 import MHDSolver
    from mhd3d_mpi_fortran_gb300.abi import Params, FP32
    pg = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        pg = dist
    n = a.n
    s, tau = workload(n)
    prm = Params(n, n, n, reconop=a.recon, stepop=2, precision=FP32, tau=tau)
    graph = not a.no_graph
    solver = MHDSolver(prm, s)
    # launch shapes: the autotuner times its compiled variants on this grid
    # (state untouched, results bit-identical), outside the timed region
    if a.tiles:
        tiles = tuple(int(t) for t in a.tiles.split(","))
        solver.set_tiles(*tiles)
    else:
        tiles = solver.autotune(reps=5)
    # warm-up (>= 3 steps), then the timed region
    solver.time_steps(max(3, a.warmup), graph=graph)
    if a.profile_only:
        solver.time_steps(2, graph=False)
        solver.close()
        return
    # e2e through the C ABI with host buffers (before the clock sampler starts)
    e2e = None
    if not a.no_e2e and rank == 0:
        e2e = e2e_run(prm, s, n, a.steps)
    if pg:
        pg.barrier()
    with Clocks(0 if ws == 1 else local) as ck:
        ms = solver.time_steps(a.steps, graph=graph)
    clocks = ck.summary()
    ms = job_time_ms(ms, pg)
    zu = whole_job_rate(n, a.steps, ws, ms)
    # per-family device time (events on the solver's stream)
    kprof = min(a.steps, 20)
    solver.set_profiling(True)
    solver.step_async(kprof)
    fam = solver.timings()
    solver.set_profiling(False)
    _, st = solver.step(1)
    stages = 2 * kprof
    fam_ms = {k: v / stages for k, v in fam.items()}  # per stage
    dom = max(WORDS, key=lambda k: fam_ms[k])
    hbm, peak_kind = peaks()
    nl = LAUNCHES[dom] + (1 if dom == "emf" and tiles[1] == 1 else 0)
    bytes_per_launch = WORDS[dom] * 4 * n ** 3 / nl
    launch_s = fam_ms[dom] * 1e-3 / nl
    achieved = bytes_per_launch / launch_s / 1e9
    traffic, traffic_prov = None, None
    tdat, traffic_prov = profile_file("traffic.json")
    if tdat is not None:
        traffic = tdat.get("per_launch", tdat).get(dom)
    solver.close()
    study = None
    if not a.no_study and rank == 0 and ws == 1:
        # the same workload in all-FP64 mode (the reference's precision) and
        # the error at equal GPU time (BASELINE's second metric), after the
        # timed region: FP64 n^3 is the reference solution of the table
        from mhd3d_mpi_fortran_gb300 import studies
        study = studies.equal_time(n=n, steps=a.study_steps, recon=a.recon)
    ens = None
    if a.ensemble_key > 0 and rank == 0 and ws == 1:
        ens = ensemble_measure(a.ensemble_key, min(a.steps, 20), a.warmup)
    cpu = None
    if not a.no_cpu_baseline and rank == 0 and ws == 1:
        v, dt, cores = cpu_rate(160, 8, a.recon)
        cpu = {"value": v, "unit": "zone-updates/s", "cores": cores, "kind": "port",
               "sample": f"8 RK2 steps of the 160^3 turbulence state (same generator), PDM, FP64 oracle "
                         f"(array passes), {dt:.1f} s",
               "detail": cpu_detail(a.recon)}
    if rank != 0:
        return
    compute_roofs = roofs(zu / ws, clocks, a.recon, tiles)
    emf_launches = 4 if tiles[1] == 1 else 3  # slice streams: three families plus their boundary rows
    # per RK2 step: the tau selection (the CFL dt comes from the previous step's
    # last stage), then per stage EMF, x faces, y and z sweeps, CT + bxyz + vf
    # and the ghost shell
    launches_per_step = 1 + 2 * (emf_launches + 3 + 1 + 1)
    fp64 = None
    if study:
        ref = study["runs"][0]
        fp64 = {"value": n ** 3 * ref["steps"] / (ref["gpu_ms"] * 1e-3), "unit": "zone-updates/s",
                "ms_per_step": ref["gpu_ms"] / ref["steps"], "steps": ref["steps"],
                "how": "the same workload in all-FP64 mode (FP64 state, fluxes and reconstructions; the "
                       "reference's precision), CUDA events around graph replays"}
    line = {
        "metric": "zone-updates/s", "value": zu, "unit": "zone-updates/s", "n_gpus": ws,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": ms / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic: seeded Gaussian-random solenoidal turbulence, k^-2 on 2<=k<=8, 256^3 periodic",
        "config": bench_config(n, a.recon),
        "launch": {"precision": "FP32 state/fluxes, FP64 metric and sums", "graph": graph,
                   "tiles": {"face_tile_len": tiles[0], "ei_emf_tile": tiles[1]},
                   "parallelism": "replicas" if ws > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, "traffic_provenance": traffic_prov,
                     "peak_kind": peak_kind},
        "hbm_roofline_160B": {"achieved_gbs": zu * 160 / 1e9 / ws, "peak": hbm, "frac": zu * 160 / 1e9 / ws / hbm,
                              "note": "compulsory 160 B per FP32 RK2 zone-update"},
        "family_ms_per_stage": fam_ms,
        **compute_roofs,
        "gpu_launches": launches_per_step * a.steps,
        "clocks": clocks,
        "status": st,
        "e2e": e2e,
        "fp64": fp64,
        "equal_time": study,
        "ensemble": ens,
        "cpu_baseline": cpu,
    }
    print(json.dumps(line), flush=True)


def ensemble_members(ngrids: int, seed: int = 0):
    """Seeded draw of the ensemble: side N uniform in {32,48,64,96}, velocity
    amplitude U[0.5,1.5], plasma beta U[0.1,10] (beta scales the OT pressure,
    whose beta is 10/3 at beta_scale 1)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = rng.choice([32, 48, 64, 96], size=ngrids)
    amp = rng.uniform(0.5, 1.5, size=ngrids)
    beta = rng.uniform(0.1, 10.0, size=ngrids)
    return [(int(n), float(a_), float(b_) / (10.0 / 3.0)) for n, a_, b_ in zip(sizes, amp, beta)]


def ensemble_measure(ngrids: int, steps: int, warmup: int) -> dict:
    """The batched ensemble (mhd_ensemble_step: one CUDA graph, one launch per
    kernel family over all grids) against the same grids stepped one after
    another (each grid's own k-step graph), both device-timed with CUDA
    events (mhd_ensemble_time, mhd_time_steps)."""
    from mhd3d_mpi_fortran_gb300 import MHDSolver, ics, ensemble_step, ensemble_autotune, ensemble_time
    from mhd3d_mpi_fortran_gb300.abi import Params, FP32
    members = ensemble_members(ngrids)
    solvers, zones = [], 0
    try:
        for i, (n, amp, bs) in enumerate(members):
            st = ics.orszag_tang_3d(n, seed=i, amp=amp, beta_scale=bs)
            solvers.append(MHDSolver(Params(n, n, n, precision=FP32, tau=0.5 * ics.cfl_dt(st)), st))
            zones += n ** 3
        tiles = ensemble_autotune(solvers, reps=3)
        ensemble_step(solvers, max(3, warmup))
        ensemble_time(solvers, steps)  # the k-step graph is captured on its first use
        ms_ens = ensemble_time(solvers, steps)
        ms_seq = 0.0
        for sv in solvers:
            sv.time_steps(steps, graph=True)  # capture and warm each grid's own k-step graph
            ms_seq += sv.time_steps(steps, graph=True)
    finally:
        for sv in solvers:
            sv.close()
    sizes = sorted({m[0] for m in members})
    return {"metric": "zone-updates/s (batched ensemble)", "value": zones * steps / (ms_ens * 1e-3),
            "unit": "zone-updates/s", "steps": steps, "ms_per_step": ms_ens / steps, "zones_per_step": zones,
            "workload": f"{ngrids} periodic 3-D Orszag-Tang grids, N uniform in {sizes}, amplitude U[0.5,1.5], "
                        f"beta U[0.1,10], PDM + RK2, FP32",
            "tiles": {"face_tile_len": tiles[0], "ei_emf_tile": tiles[1]},
            "sequential": {"value": zones * steps / (ms_seq * 1e-3), "ms_per_step": ms_seq / steps,
                           "how": "each grid's own k-step CUDA graph, one grid after another"},
            "timing": "CUDA events on the ensemble's stream around its graph (device time)"}


def run_ensemble(a):
    line = ensemble_measure(a.ensemble, a.steps, a.warmup)
    line.update({"n_gpus": 1, "warmup": a.warmup, "higher_is_better": True, "dtype": "f32",
                 "data": "synthetic: seeded OT ensemble"})
    print(json.dumps(line), flush=True)


def main():
    a = parse()
    if a.ingest_counts:
        ingest_counts(a)
        return
    if a.ensemble:
        run_ensemble(a)
        return
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
