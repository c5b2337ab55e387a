#!/usr/bin/env python3
"""Benchmark: WRF-ARW physics-off large step (solve_em RK3 + acoustic steps).

Metric: cell-steps/s (one mass cell advanced one full large step: 3 RK
stages, all acoustic sub-steps and all scalars); cells = (ide-1)(jde-1)(kde-1).

Default workload (one GPU): 512 x 512 x 80 levels, dx = 1 km, dt = 6 s,
sixteen +3 K bubbles, qv + 10 positive-definite passive scalars, FP32, the
plain single-domain form (the drop-in).  Seeded synthetic initial state
(Weisman-Klemp sounding); the device state (~6 GB) is far larger than L2.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload c2|c1|c3|c4|c5] [--mixed]

N > 1 runs N independent replicas (one per rank, no collective on the data
path) and reports the whole-job rate; the reference arm times the CPU
restatement of the reference on the host cores (rank 0 only).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HBM_FALLBACK_GBS = 6800.0


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return HBM_FALLBACK_GBS, "fallback"


# Algorithmic bytes per mass cell and large step of each kernel family:
# unique 3-D FP32 arrays read + written by the routine(s) it implements
# (2-D and 1-D arrays ignored) x 4 B x its launches per step (3 RK stages,
# 7 acoustic steps with 4 sound steps per step).  s_pd / s_all: species
# advected by the positive-definite scheme / all species.
def alg_bytes_per_cell_step(phase, s_pd, s_all, n_acoustic=7):
    s_np = s_all - s_pd
    per = {
        "step_prep": 3 * (8 + 9),          # u v w ph phb al alb qv -> ru rv rw ww php alt cqu cqv cqw
        "rk_tend_u": 3 * (12 + 1),         # u ru rv rw ww ph alt p pb al php cqu (+v) -> ru_tend
        "rk_tend_v": 3 * (12 + 1),
        "rk_tend_w": 3 * (8 + 2),          # w ru rv ww p cqw u v -> rw_tend, cqw
        "rk_tend_t": 3 * (5 + 1),          # t ru rv ww -> t_tend
        "rk_tend_ph": 3 * (7 + 1),         # u v ww ph phb w -> ph_tend
        "cfl_check": 3 * 5,
        "small_step_prep": 3 * (16 + 13),
        "calc_p_rho_0": 3 * (7 + 3),
        "calc_coef_w": 3 * (2 + 3),
        "advance_uv": n_acoustic * (14 + 2),
        "advance_mu_t": n_acoustic * (9 + 3),
        "advance_w": n_acoustic * (17 + 3),
        "sumflux_calc_p_rho": n_acoustic * (13 + 6),
        "small_step_finish": 3 * (13 + 6),
        "rk_update_scalar_pd": 2 * s_pd,
        # stages 1-2: read q (+ q_old at stage 2), write new q (+ q_old at stage 1),
        # mass fluxes once; stage 3: the species not using the PD scheme
        "scalar_adv_update": 2 * (3 * s_all + 3) + ((3 * s_np + 3) if s_np else 0),
        "scalar_pd_update": (3 * s_pd + 3) if s_pd else 0,
        "calc_p_rho_phi": 3 * (6 + 2),
        "set_w_surface": 0,
        "bc_fill": 0,
    }
    return 4 * per.get(phase, 0)


# Contract bytes per cell-step: unique 3-D arrays read plus written between
# the reference's global sync points of one large step (halo exchanges and
# boundary fills of solve_em), N = 553 + 3 n_moist + 8 S array passes of 4 B
# with S species in all (qv included), plus 4 B per access of each array the
# mixed form keeps in FP64 (a, alpha, gamma: 30 accesses).  Re-reads between
# kernels that the reference would also do between its own loops are not
# counted, so this is the floor a fully fused step could reach.
def contract_bytes_per_cell_step(n_moist, n_species, mixed=False):
    return 4 * (553 + 3 * n_moist + 8 * n_species) + (120 if mixed else 0)


# DRAM bytes (read + write) per mass cell of one launch, from the ncu
# captures summarised in profiles/ (256x256x80 case, inputs far larger than
# L2; traffic grows with the cells processed, so it scales to other sizes):
# the capture of k_scalar_pd_update, of k_scalar_adv_update (stage 1) and of
# the acoustic column kernels.
NCU_DRAM_BYTES_PER_CELL = {
    "scalar_pd_update": 1032.8e6 / 5177344,
    "scalar_adv_update": 780.6e6 / 5177344,
    "advance_w": 451.3e6 / 5177344,
}

PHASE_NAMES = ["step_prep", "rk_tend_u", "rk_tend_v", "rk_tend_w", "rk_tend_t", "rk_tend_ph", "cfl_check",
               "small_step_prep", "calc_p_rho_0", "calc_coef_w", "advance_uv", "advance_mu_t", "advance_w",
               "sumflux_calc_p_rho", "small_step_finish", "rk_update_scalar_pd", "scalar_adv_update",
               "scalar_pd_update", "calc_p_rho_phi"]


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.rows = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if self.t:
            self.t.join(timeout=5)
        sm = []
        smax = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                smax = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_case(workload, nx=None):
    from wrf_gb300 import cases
    if workload == "c1":
        return cases.config1()
    if workload == "c2":
        return cases.config2() if not nx else cases.config2(nx=nx)
    if workload == "c3":
        return cases.config3() if not nx else cases.config3(nx=nx)
    raise ValueError(workload)


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def allreduce_max(pg, x):
    from wrf_gb300.replicas import reduce_max
    return reduce_max(pg, x)


def run_reference(args, world, rank):
    """Reference arm: the CPU restatement of the reference's solve_em path on
    the host cores (all threads), same workload / metric."""
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _harness import OracleDomain
    case = make_case(args.workload, args.nx)
    cores = os.cpu_count() or 1
    od = OracleDomain(case, "f32", nthreads=cores)
    # one warm-up step (also sizes the sample), then the same K steps as the
    # GPU arm unless they would exceed the time budget
    t0 = time.perf_counter()
    od.step(1)
    t_step = time.perf_counter() - t0
    steps = args.steps if args.ref_steps is None else args.ref_steps
    steps = max(1, min(steps, int(args.ref_budget_s / max(t_step, 1e-3))))
    t0 = time.perf_counter()
    od.step(steps)
    el = time.perf_counter() - t0
    val = case.cells() * steps / el
    sample = "%d of the %d timed steps of the %s workload (after 1 warm-up step; budget %.0f s), " \
             "%d OpenMP threads" % (steps, args.steps, case.name, args.ref_budget_s, cores)
    line = {
        "impl": "reference", "metric": "cell-steps/s", "value": val, "unit": "cell-steps/s",
        "n_gpus": args.gpus, "steps": steps, "warmup": 1, "ms_per_step": 1e3 * el / steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded Weisman-Klemp supercell state)",
        "config": {"workload": case.name, "global_batch": 1, "seq_len": None, "parallelism": "cpu-openmp",
                   "l2": "state larger than L2"},
        "cpu_baseline": {"value": val, "unit": "cell-steps/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline(case, seconds_budget=25.0, max_steps=10):
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from _harness import OracleDomain
    cores = os.cpu_count() or 1
    od = OracleDomain(case, "f32", nthreads=cores)
    t0 = time.perf_counter()
    od.step(1)
    el1 = time.perf_counter() - t0
    steps = 1
    if el1 < seconds_budget / 3:
        n = max(1, int((seconds_budget - el1) / max(el1, 1e-3)))
        n = min(n, max_steps)
        t0 = time.perf_counter()
        od.step(n)
        el1 = (time.perf_counter() - t0) / n
        steps = n
    return {"value": case.cells() / el1, "unit": "cell-steps/s", "cores": cores, "kind": "port",
            "sample": "%d large step(s) of the %s workload after one warm-up step, %d OpenMP threads (CPU restatement "
                      "of the reference's FP32 solve_em path)" % (steps, case.name, cores)}


def _copy_member_state(src, ms, dst, md, nsp):
    """Copy every field of member ms of one ensemble into member md of
    another (same domain description), through host memory."""
    from wrf_gb300 import abi
    ids = list(abi.FIELD_ID.values()) + [abi.species_id(s) for s in range(nsp)] + \
        [abi.species_id(s, True) for s in range(nsp)]
    for fid in ids:
        if src.field_size(ms, fid) > 0:
            dst.set(md, fid, src.get(ms, fid))


def ensemble_accuracy(n_members=2, steps=(1, 10, 30, 60)):
    """FP64-oracle error of the batched mixed form (and of the plain FP32
    form and the FP32 oracle) on the smallest members of the uneven
    ensemble, after each of `steps` large steps."""
    from wrf_gb300 import cases
    specs = cases.ensemble_members(seed=4)
    order = sorted(range(len(specs)), key=lambda q: specs[q][0] * specs[q][1] * specs[q][2])[:n_members]
    res = accuracy_vs_fp64([cases.ensemble_member(specs[q]) for q in order], steps)
    res["members"] = res.pop("cases")
    return res


def accuracy_vs_fp64(mcases, steps=(1, 10, 30, 60), names=("u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al")):
    """diffwrf relative L2 (serr) per field of the GPU plain FP32 form, the
    GPU mixed form and the FP32 oracle (the reference's own arithmetic)
    against the FP64 oracle, all from the same FP32-rounded initial state,
    after each of `steps` large steps; fields of several cases are pooled."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import numpy as np
    from _harness import OracleDomain, interior, serr
    from wrf_gb300 import abi
    from wrf_gb300 import gpu as G
    cores = os.cpu_count() or 1
    o64 = [OracleDomain(c, "f64", nthreads=cores, load=False) for c in mcases]
    for c, o in zip(mcases, o64):
        for fid, arr in c.field_items():
            o.set(fid, arr, as_f32=True)
    o32 = [OracleDomain(c, "f32", nthreads=cores) for c in mcases]
    mixed = G.Ensemble.from_cases(mcases, flags=G.FLAG_MIXED)
    plain = G.Ensemble.from_cases(mcases, flags=0)
    out = {"cases": [c.name for c in mcases], "oracle": "FP64 restatement, same FP32-rounded initial state",
           "serr": {}}
    done = 0
    for n in steps:
        for o in o64 + o32:
            o.step(n - done)
        mixed.step(n - done)
        plain.step(n - done)
        done = n
        mixed.sync()
        plain.sync()
        row = {}
        getters = (("mixed", lambda m, c, f: mixed.get(m, f)), ("plain", lambda m, c, f: plain.get(m, f)),
                   ("oracle_f32", lambda m, c, f: o32[m].get(f)))
        for label, get in getters:
            row[label] = {}
            for nm in list(names) + ["qv"]:
                fid = abi.species_id(0) if nm == "qv" else abi.FIELD_ID[nm]
                a = [interior(c, fid, get(m, c, fid)) for m, c in enumerate(mcases)]
                b = [interior(c, fid, o.get(fid)) for c, o in zip(mcases, o64)]
                row[label][nm] = float(serr(np.concatenate([x.ravel() for x in a]),
                                            np.concatenate([x.ravel() for x in b])))
        out["serr"][str(n)] = row
    mixed.close()
    plain.close()
    return out


def c3_accuracy(nx=128, kde=96):
    """The C3 precision configuration's accuracy against the FP64 oracle:
    the f-plane jet channel at nx x nx x kde (dx = 4 km, dt = 20 s, top 25 km;
    the full 1024 x 1024 channel's FP64 run would take tens of minutes on the
    host), after 1, 10, 30 and 60 steps."""
    from wrf_gb300 import cases
    c = cases.config3(nx=nx, kde=kde)
    res = accuracy_vs_fp64([c])
    res["size"] = "%dx%dx%d (the 1024x1024x96 channel's dx, dt, levels and jet; narrower channel)" % (nx, nx, kde)
    return res


def ensemble_bench(steps, warmup, n_members=64, world=1, rank=0, pg=None):
    """Uneven 64-member ensemble (nx, ny ~ U[64, 256], 41..80 levels, 3 PD
    scalars, dx = 2 km, dt = 12 s): cell-steps/s of the batched forms (all
    members in one graph-captured step, FP32 and mixed FP32 + FP64 columns)
    and of the plain single-domain form run member after member.  With N
    ranks the members are sharded by size (no collective on the data path)
    and the rates are whole-job: all ranks' cells / the slowest rank's time."""
    from wrf_gb300 import cases
    from wrf_gb300 import gpu as G
    from wrf_gb300.replicas import shard_members, job_rate
    all_specs = cases.ensemble_members(seed=4)[:n_members]
    all_descs = [cases.ensemble_member_desc(s) for s in all_specs]
    all_cells = [(d.ide - 1) * (d.jde - 1) * (d.kde - 1) for d in all_descs]
    mine = shard_members(all_cells, world)[rank]
    specs = [all_specs[q] for q in mine]
    descs = [all_descs[q] for q in mine]
    cells = sum(all_cells[q] for q in mine)
    nsp = descs[0].n_moist + descs[0].n_scalar
    t0 = time.perf_counter()
    ens = G.Ensemble(descs, flags=G.FLAG_MIXED)
    for m, sp in enumerate(specs):
        ens.load_case(m, cases.ensemble_member(sp))
    build_s = time.perf_counter() - t0
    tune_mixed = ens.autotune(2)
    res = {"workload": "c4_ensemble_%d_members" % len(all_specs), "cells": sum(all_cells), "species": nsp,
           "members": len(all_specs), "members_per_rank": [len(x) for x in shard_members(all_cells, world)],
           "state_build_s": round(build_s, 1), "device_gb_mixed": round(ens.device_bytes() / 1e9, 2),
           "tuning_mixed": {f: t["param"] for f, t in tune_mixed.items()}}
    ens.step(warmup)
    ens.sync()
    barrier(pg)
    ms = ens.time_steps(steps)
    res["batched_mixed"], _, slow = job_rate(pg, cells * steps, ms / 1e3)
    res["batched_mixed_ms_per_step"] = 1e3 * slow / steps
    res["batched_mixed_phases_ms"] = {k: round(v[0], 3) for k, v in ens.profile_phases(1).items()}
    # batched FP32: same members, same state
    f32 = G.Ensemble(descs, flags=0)
    for m in range(len(specs)):
        _copy_member_state(ens, m, f32, m, nsp)
    f32.autotune(2)
    f32.step(warmup)
    f32.sync()
    barrier(pg)
    ms32 = f32.time_steps(steps)
    res["batched_f32"], _, _ = job_rate(pg, cells * steps, ms32 / 1e3)
    res["batched_f32_phases_ms"] = {k: round(v[0], 3) for k, v in f32.profile_phases(1).items()}
    f32.close()
    # plain single-domain form: every member alone, one after another
    tot_ms = 0.0
    for m, d in enumerate(descs):
        dom = G.Ensemble([d], flags=0)
        _copy_member_state(ens, m, dom, 0, nsp)
        dom.autotune(1)
        dom.step(warmup)
        dom.sync()
        tot_ms += dom.time_steps(steps)
        dom.close()
    res["plain_sequential"], _, slow = job_rate(pg, cells * steps, tot_ms / 1e3)
    res["plain_ms_per_step"] = 1e3 * slow / steps
    res["batched_mixed_over_plain"] = res["batched_mixed"] / res["plain_sequential"]
    ens.close()
    return res


def _build_c5_member(spec):
    """Worker (spawned process): one C5 member's initial state, FP32 arrays."""
    sys.path.insert(0, ROOT)
    from wrf_gb300 import cases
    c = cases.c5_member(spec)
    return [(fid, a.astype("float32")) for fid, a in c.field_items()]


def c5_buckets(specs, nbuckets=3):
    """Members sorted by cell count and cut into nbuckets groups of about
    equal total cells (small, medium, large members)."""
    cells = [sp[1] * sp[2] * (sp[3] - 1) for sp in specs]
    order = sorted(range(len(specs)), key=lambda q: cells[q])
    total = float(sum(cells))
    out, cur, acc = [], [], 0.0
    for q in order:
        cur.append(q)
        acc += cells[q]
        if acc >= total * (len(out) + 1) / nbuckets and len(out) < nbuckets - 1:
            out.append(cur)
            cur = []
    out.append(cur)
    return out


def run_c5_line(args, world, rank, local, pg):
    """--workload c5: 256 uneven members (supercell and jet-channel states
    mixed, qv + 7 PD scalars each, FP32 bulk with FP64 column steps).  The
    whole ensemble's state (~1e9 cells, ~360 GB as laid out here) is larger
    than one GB300's memory, so the members run in three size buckets of
    about equal cells, each bucket one batched graph-captured ensemble;
    value = all cells x steps / the buckets' summed time.  Per bucket: cell-
    steps/s, and the FP64-oracle error of its smallest supercell and channel
    members after 1, 10, 30, 60 and 120 steps."""
    import concurrent.futures as cf
    import multiprocessing as mp
    from wrf_gb300 import cases
    from wrf_gb300 import gpu as G
    specs = cases.c5_members()
    buckets = c5_buckets(specs)
    # member states are built by spawned workers (started before any CUDA work here)
    pool = cf.ProcessPoolExecutor(max_workers=max(1, min(16, (os.cpu_count() or 2) - 1)),
                                  mp_context=mp.get_context("spawn"))
    sampler = ClockSampler(local)
    res = {"workload": "c5_mixed_256_members", "members": len(specs),
           "cells": sum(sp[1] * sp[2] * (sp[3] - 1) for sp in specs), "buckets": []}
    tot_cells_steps = 0.0
    tot_s = 0.0
    sampler.start()
    for b, members in enumerate(buckets):
        mspecs = [specs[q] for q in members]
        descs = [cases.c5_member_desc(sp) for sp in mspecs]
        t0 = time.perf_counter()
        ens = G.Ensemble(descs, flags=G.FLAG_MIXED)
        # states stream in as the workers finish them (host memory stays bounded)
        for m, fields in enumerate(pool.map(_build_c5_member, mspecs, chunksize=1)):
            for fid, arr in fields:
                ens.set(m, fid, arr)
        build_s = time.perf_counter() - t0
        ens.autotune(1)
        ens.step(args.warmup)
        ens.sync()
        bcells = sum(sp[1] * sp[2] * (sp[3] - 1) for sp in mspecs)
        ms = ens.time_steps(args.steps)
        dev_gb = ens.device_bytes() / 1e9
        ens.close()
        tot_cells_steps += bcells * args.steps
        tot_s += ms / 1e3
        res["buckets"].append({
            "members": len(mspecs), "channel_members": sum(sp[0] == "channel" for sp in mspecs),
            "cells": bcells, "cells_per_member": [min(sp[1] * sp[2] * (sp[3] - 1) for sp in mspecs),
                                                  max(sp[1] * sp[2] * (sp[3] - 1) for sp in mspecs)],
            "device_gb": round(dev_gb, 1), "state_build_s": round(build_s, 1),
            "ms_per_step": ms / args.steps, "cell_steps_per_s": bcells * args.steps / (ms / 1e3)})
    clocks = sampler.stop()
    pool.shutdown()
    value = tot_cells_steps / tot_s
    # accuracy: the smallest supercell and channel member of every bucket
    acc_steps = (1, 10, 30, 60, 120)
    for b, members in enumerate(buckets):
        picks = []
        for kind in ("supercell", "channel"):
            ks = [q for q in members if specs[q][0] == kind]
            if ks:
                picks.append(min(ks, key=lambda q: specs[q][1] * specs[q][2] * specs[q][3]))
        try:
            acc = accuracy_vs_fp64([cases.c5_member(specs[q]) for q in picks], acc_steps)
        except Exception as ex:  # reported, never required
            acc = {"error": repr(ex)}
        res["buckets"][b]["accuracy"] = acc
    hbm, hbm_kind = peaks()
    alg = contract_bytes_per_cell_step(1, 8, mixed=True)
    line = {
        "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64-columns",
        "data": "synthetic (seeded supercell and f-plane jet-channel members, uneven sizes)",
        "config": {"workload": res["workload"], "form": "batched+mixed, three size buckets run one after another",
                   "cells": res["cells"], "global_batch": len(specs), "seq_len": None, "parallelism": "single",
                   "l2": "inputs larger than L2"},
        "roofline": {"bound": "hbm", "achieved": alg * value / 1e9, "peak": hbm, "peak_kind": hbm_kind,
                     "unit": "GB/s", "frac": alg * value / 1e9 / hbm, "traffic": None,
                     "note": "whole step at the contract bytes per cell-step (%d B) x cell-steps/s" % alg},
        "c5": res, "clocks": clocks,
    }
    print(json.dumps(line), flush=True)


def run_ensemble_line(args, world, rank, local, pg):
    """--workload c4: the uneven 64-member ensemble on its own line (value =
    batched mixed form), with the plain sequential form and the FP64 error."""
    sampler = ClockSampler(local)
    sampler.start()
    res = ensemble_bench(args.steps, args.warmup, world=world, rank=rank, pg=pg)
    clocks = sampler.stop()
    hbm, hbm_kind = peaks()
    alg = contract_bytes_per_cell_step(1, 4, mixed=True)
    acc = ensemble_accuracy() if rank == 0 else None
    if rank == 0:
        line = {
            "metric": "cell-steps/s", "value": res["batched_mixed"], "unit": "cell-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["batched_mixed_ms_per_step"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64-columns",
            "data": "synthetic (seeded Weisman-Klemp supercell members, uneven sizes)",
            "config": {"workload": res["workload"], "form": "batched+mixed", "cells": res["cells"],
                       "global_batch": res["members"], "seq_len": None,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (%.1f GB device state)" % res["device_gb_mixed"]},
            "roofline": {"bound": "hbm", "achieved": alg * res["batched_mixed"] / 1e9, "peak": hbm,
                         "peak_kind": hbm_kind, "unit": "GB/s",
                         "frac": alg * res["batched_mixed"] / 1e9 / hbm, "traffic": None,
                         "note": "whole step at the contract bytes per cell-step (%d B: unique arrays between the "
                                 "reference's sync points, FP64 a/alpha/gamma included) x cell-steps/s" % alg},
            "ensemble": res, "accuracy": acc, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=["c1", "c2", "c3", "c4", "c5"])
    ap.add_argument("--no-c3-accuracy", action="store_true",
                    help="skip the C3 channel's FP64-oracle accuracy block")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the uneven-ensemble comparison (batched+mixed vs plain) added to the default line")
    ap.add_argument("--mixed", action="store_true", help="mixed-precision form (FP64 column steps)")
    ap.add_argument("--nx", type=int, default=None, help="horizontal size of the supercell workload (profiling runs)")
    ap.add_argument("--ref-steps", type=int, default=None,
                    help="reference arm: steps to time (default: the same --steps as the GPU arm, within the budget)")
    ap.add_argument("--ref-budget-s", type=float, default=150.0,
                    help="reference arm: time budget of the timed steps (seconds)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-open", action="store_true",
                    help="skip the same workload with open lateral boundaries added to the default line")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--tune-rounds", type=int, default=2,
                    help="autotuning rounds before the warm-up (0: default launch variants; profiling runs)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup

    world, rank, local, pg = dist_setup(args)
    try:
        if args.impl == "reference":
            run_reference(args, world, rank)
        elif args.workload == "c4":
            run_ensemble_line(args, world, rank, local, pg)
        elif args.workload == "c5":
            run_c5_line(args, world, rank, local, pg)
        else:
            run_single(args, world, rank, local, pg)
    finally:
        if pg is not None:
            pg.destroy_process_group()


def run_single(args, world, rank, local, pg):
    """One domain per rank (replicas for N > 1): the default line."""
    from wrf_gb300 import abi
    from wrf_gb300 import gpu as G
    case = make_case(args.workload, args.nx)
    flags = G.FLAG_MIXED if args.mixed else 0
    dom = G.Domain(case, flags=flags)
    cells = case.cells()
    # online autotuning of the launch variants (advances the model 4 x rounds steps)
    tuning = dom.autotune(args.tune_rounds) if args.tune_rounds > 0 else dom.tuning()

    # warm-up (also builds the CUDA graph)
    dom.step(args.warmup)
    dom.sync()
    rc, bits, vcfl, hcfl = dom.status(0)
    if rc != 0:
        raise SystemExit("health check failed after warm-up: rc=%d bits=%d" % (rc, bits))

    # timed region: K steps, device events on the library's stream
    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    barrier(pg)
    dom.sync()
    ms = dom.time_steps(args.steps)
    barrier(pg)
    clocks = sampler.stop()
    ms = allreduce_max(pg, ms)
    value = cells * args.steps * world / (ms / 1e3)

    dev_gb = dom.device_bytes() / 1e9
    # per-kernel phases (events between launches, outside the timed region)
    phases = dom.profile_phases(1)
    launches = dom.launches_per_step()
    hbm, hbm_kind = peaks()
    nsp = case.desc.n_moist + case.desc.n_scalar
    s_pd = (1 if case.desc.config.moist_adv_opt == 1 else 0) + (case.desc.n_scalar if case.desc.config.scalar_adv_opt == 1 else 0)
    alg = {k: alg_bytes_per_cell_step(k, s_pd, nsp) * cells for k in phases}
    dom_name = max((k for k in phases if alg[k] > 0), key=lambda k: phases[k][0])
    dom_ms, dom_n = phases[dom_name]
    achieved = alg[dom_name] / (dom_ms / 1e3) / 1e9
    step_alg = sum(alg.values())
    step_ms = ms / args.steps
    contract = contract_bytes_per_cell_step(case.desc.n_moist, nsp, args.mixed) * cells
    traffic = None
    if dom_name in NCU_DRAM_BYTES_PER_CELL and case.desc.n_scalar == 10:
        traffic = NCU_DRAM_BYTES_PER_CELL[dom_name] * cells
    roofline = {"bound": "hbm", "kernel": dom_name, "achieved": achieved, "peak": hbm, "peak_kind": hbm_kind,
                "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
                "traffic_note": "DRAM bytes per launch from the ncu capture of the 256x256x80 case, scaled by cells",
                "alg_bytes_per_step": alg[dom_name], "ms_per_step": dom_ms, "launches_per_step": dom_n,
                "step_contract_bytes": contract, "step_achieved": contract / (step_ms / 1e3) / 1e9,
                "step_frac": contract / (step_ms / 1e3) / 1e9 / hbm,
                "step_frac_note": "whole step at the contract bytes (unique arrays between the reference's sync "
                                  "points: %d B per cell-step)" % (contract // cells),
                "step_kernel_bytes": step_alg, "step_kernel_frac": step_alg / (step_ms / 1e3) / 1e9 / hbm,
                "step_kernel_note": "whole step at the sum of every kernel's own unique arrays (%d B per "
                                    "cell-step; counts re-reads between kernels)" % (step_alg // cells),
                "note": "frac of %s HBM copy bandwidth; kernel times from CUDA events between launches" % hbm_kind}

    # end to end through the C ABI with host buffers (pinned)
    e2e = None
    if not args.no_e2e:
        import numpy as np
        try:
            import torch
            pin = lambda n: torch.empty(n, dtype=torch.float32, pin_memory=True).numpy()
        except Exception:
            pin = lambda n: np.empty(n, dtype=np.float32)
        fids = [abi.FIELD_ID[n] for n in ("u_2", "v_2", "w_2", "t_2", "ph_2", "mu_2", "p", "al")]
        nsp = case.desc.n_moist + case.desc.n_scalar
        fids += [abi.species_id(s) for s in range(nsp)]
        bufs = {}
        for f in fids:
            n = dom.field_size(0, f)
            b = pin(n)
            b[:] = dom.get(0, f)
            bufs[f] = b
        h2d = sum(b.nbytes for b in bufs.values())
        d2h = h2d
        dom.bind_host_state(0, list(bufs), list(bufs.values()))
        dom.step_host(3)  # captures the step's graphs with their copies (first, middle, last step of a call)
        dom.sync()
        barrier(pg)
        t0 = time.perf_counter()
        dom.step_host(args.steps)
        dom.sync()
        el = allreduce_max(pg, time.perf_counter() - t0)
        dom.unbind_host_state()
        e2e = {"value": cells * args.steps * world / el, "unit": "cell-steps/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "what": "per step: H2D of the prognostic state (u,v,w,theta,ph,mu,p,al + %d species) from pinned "
                       "host memory, one large step, D2H of the same fields into the same host buffers (the next "
                       "step's input), through the C ABI (wrfgpu_step_host: the copies are nodes of the step's "
                       "graph; the passive scalars' upload overlaps stage 1's dynamics)" % nsp}

    # the same workload with open lateral boundaries on all four sides (the
    # em_quarter_ss namelist): the tile kernels plus the edge-strip
    # recomputation next to the open edges and the acoustic-step halo fills
    open_bc = None
    if args.workload == "c2" and not args.nx and not args.no_open and world == 1:
        from wrf_gb300 import cases as C
        try:
            ocase = C.open_boundaries(case)
            odom = G.Domain(ocase, flags=flags)
            if args.tune_rounds > 0:
                odom.autotune(args.tune_rounds)
            odom.step(args.warmup)
            odom.sync()
            orc = odom.status(0)[0]
            osteps = max(3, min(args.steps, 10))
            oms = odom.time_steps(osteps)
            ophases = odom.profile_phases(1)
            open_bc = {"workload": ocase.name, "sides": "open_xs/xe/ys/ye", "status": orc,
                       "ms_per_step": oms / osteps, "value": cells * osteps / (oms / 1e3), "unit": "cell-steps/s",
                       "steps": osteps, "overhead_vs_periodic": (oms / osteps) / (ms / args.steps) - 1.0,
                       "launches_per_step": odom.launches_per_step(),
                       "phase_ms_delta_vs_periodic": {k: round(ophases[k][0] - phases[k][0], 4)
                                                      for k in ophases if k in phases}}
            odom.close()
        except Exception as ex:  # reported, never required
            open_bc = {"error": repr(ex)}

    ensemble = None
    if args.workload == "c2" and not args.nx and not args.no_ensemble and world == 1:
        dom.close()
        try:
            ensemble = ensemble_bench(max(2, min(args.steps, 3)), 3)
            hbm_e, _ = peaks()
            ens_alg = contract_bytes_per_cell_step(1, 4, mixed=True)
            ensemble["step_contract_bytes_per_cell"] = ens_alg
            ensemble["batched_mixed_hbm_frac"] = ens_alg * ensemble["batched_mixed"] / 1e9 / hbm_e
            ensemble["accuracy"] = ensemble_accuracy()
        except Exception as ex:  # reported, never required
            ensemble = {"error": repr(ex)}

    c3acc = None
    if rank == 0 and world == 1 and args.workload in ("c2", "c3") and not args.nx and not args.no_c3_accuracy:
        try:
            c3acc = c3_accuracy()
        except Exception as ex:  # reported, never required
            c3acc = {"error": repr(ex)}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(case)
        except Exception as ex:  # the baseline is reported, never required
            cpu = {"error": str(ex)}

    if rank == 0:
        line = {
            "metric": "cell-steps/s", "value": value, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32" if not args.mixed else "f32+f64-columns",
            "data": ("synthetic (seeded f-plane jet channel in thermal-wind balance, +-1 K noise, qv at 80% RH)"
                     if args.workload == "c3" else
                     "synthetic (seeded Weisman-Klemp supercell state, 16 bubbles, log-normal scalars)"),
            "config": {"workload": case.name, "form": "mixed" if args.mixed else "plain",
                       "cells": cells, "species": case.desc.n_moist + case.desc.n_scalar,
                       "global_batch": world, "seq_len": None,
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (%.1f GB device state)" % (dev_gb),
                       "tuning": {f: t["param"] for f, t in tuning.items()}},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
            "gpu_launches": launches * args.steps,
            "clocks": clocks,
            "phases_ms_per_step": {k: round(v[0], 4) for k, v in phases.items()},
            "ensemble": ensemble,
            "c3_accuracy": c3acc,
            "open_boundaries": open_bc,
        }
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
