"""Benchmark: X^T X assembly throughput (rows/s) on one GB300.

Workload (default): the binary-alloy precision-path configuration - 5,000
seeded synthetic structures of 64..128 atoms (bcc/fcc supercells, a ~ U(2.8,
4.2) A, displacements N(0, 0.15 A), random A/B occupancy), Morse labels,
gtinv order 3, l_max (8, 4), 10 Gaussians + constant, cutoff 7 A,
model_type 3, max_p 2 (F = 2,618 columns, ~1.3 M rows).

One step = one pass of the hot path over the whole dataset: neighbour lists,
a_nlm, invariant features and their force/stress derivatives (X rows, FP32
features with long neighbour sums), row weighting, X^T y, and X^T X on the
tcgen05 tensor cores (the FP32 rows split into four fixed-point BF16 slices
per 1,024-row segment, 13 slice products with exact FP32 partial sums,
float-float segment sums: the Gram of the FP32 rows to ~1e-12).

  value : rows/s with the structures, weights and targets resident in HBM.
  e2e   : rows/s through the C ABI with host buffers (pg_gram_accumulate: host
          cell translations + H2D copies, then pg_gram_result: D2H of X^T X).
  cpu_baseline : the CPU oracle (the reference algorithm restated in C++,
          OpenMP over structures) + numpy X^T X on a bounded sample.
  fit   : the full ridge fit of the same workload (80/20 split of the
          structures, alphas 10^linspace(-3, 1, 5)) in mixed precision and in
          FP64: wall seconds of each phase, X^T X rows/s of each, and the
          energy / force RMSEs of the two fitted models on the test structures
          (FP64 evaluator) with their differences.
  eval  : E/F/S atoms/s of the evaluator, mixed and FP64, with its roofline
          (flops per atom from the model's work figures, nominal CUDA-core peaks).
  cfg5  : one pass over 5,000 structures of the order-4 ternary model
          (F = 21,945): rows/s, the Gram's TFLOP/s, and the ridge solve seconds
          at that size.

`--impl reference` times the reference's CPU algorithm instead (the oracle
port; the reference's own build is not available on the GPU host) on the
same workload, metric and unit, one bounded sample per step.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "X\u1d40X rows/s & E/F/S atoms/s, 1 GB300, mixed vs FP64 at \u0394RMSE<0.05 meV/atom"
UNIT = "rows/s"

CFG2 = dict(n_type=2, cutoff=7.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 10), gtinv_order=3,
            gtinv_maxl=(8, 4))
# The other configurations of the benchmark family, for `--model`: the unary
# fcc model (F = 1,539), the ternary model (F = 8,262) and the order-4 ternary
# model (F = 21,945); each with its structure generator and default size.
MODELS = {
    "cfg1": (dict(n_type=1, cutoff=6.0, model_type=2, max_p=2, gaussian_params2=(0.0, 5.0, 8), gtinv_order=2,
                  gtinv_maxl=(4,)), "fcc", 200,
             "unary fcc, 200 structures of 32 atoms, gtinv order 2, l_max 4, 8+1 Gaussians, rc 6 A, model_type 2"),
    "cfg2": (CFG2, "binary", 5000,
             "binary alloy, 5000 structures of 64-128 atoms, gtinv order 3, l_max (8,4), 10+1 Gaussians, rc 7 A, "
             "model_type 3, max_p 2"),
    "cfg3": (dict(n_type=3, cutoff=6.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 8), gtinv_order=3,
                  gtinv_maxl=(6, 4)), "ternary", 20000,
             "ternary, random triclinic cells of 8-256 atoms, gtinv order 3, l_max (6,4), 8+1 Gaussians, rc 6 A, "
             "model_type 3, max_p 2"),
    "cfg5": (dict(n_type=3, cutoff=8.0, model_type=3, max_p=2, gaussian_params2=(0.0, 5.0, 4), gtinv_order=4,
                  gtinv_maxl=(8, 8, 2)), "ternary32", 50000,
             "ternary, random triclinic cells of 32-192 atoms, gtinv order 4, l_max (8,8,2), 4+1 Gaussians, rc 8 A, "
             "model_type 3, max_p 2"),
}


# DRAM traffic of pg_rows_pairs per X row, from one ncu capture (binary model,
# mixed precision, 20 structures, 5,552 rows: dram__bytes_read.sum 0.282 GB +
# dram__bytes_write.sum 1.497 GB).  The kernel's traffic is the group vectors it
# writes, which grow with the pair images, in proportion to the rows; the bench
# line scales it to a launch by the rows the launch processes.
NCU_ROWS_PAIRS_BYTES_PER_ROW = {"cfg2": (0.291940 + 1.483896) * 1e9 / 5552}


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def dist_env():
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), int(
        os.environ.get("LOCAL_RANK", "0"))


def make_dataset(n_struct, seed, device, kind="binary", rc=7.0):
    from pypolymlp_gb300 import synthetic as syn
    from pypolymlp_gb300.regression import Dataset

    if kind == "fcc":
        ss, nt = syn.fcc_set(n_struct, seed=seed), 1
    elif kind == "ternary":
        ss, nt = syn.ternary_set(n_struct, seed=seed), 3
    elif kind == "ternary32":
        ss, nt = syn.ternary_set(n_struct, seed=seed, n_range=(32, 192)), 3
    else:
        ss, nt = syn.binary_set(n_struct, seed=seed), 2
    t = time.time()
    syn.morse_labels(ss, syn.morse_D(nt), rc=rc, device=device)
    log(f"labels for {n_struct} structures in {time.time() - t:.1f}s")
    return Dataset.from_structure_set(ss, name="binary")


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.path = tempfile.mktemp(suffix=".csv")
        self.proc = None
        self.gpu = gpu_index

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        sm, mx, reasons = [], [], set()
        try:
            with open(self.path) as f:
                for line in f:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) < 9:
                        continue
                    try:
                        sm.append(float(p[1]))
                        mx.append(float(p[2]))
                    except ValueError:
                        continue
                    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
                    for name, v in zip(names, p[5:9]):
                        if v.lower().startswith("active"):
                            reasons.add(name)
        except OSError:
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    path = os.path.join(HERE, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    return 6800.0, 1900.0, "fallback"


def cpu_baseline(params, data, sample, n_threads):
    """CPU oracle (reference algorithm) + numpy Gram on the first `sample` structures."""
    from oracle.pipeline import calc_xtx_xty_cpu
    from pypolymlp_gb300.regression import get_min_energy

    sub = data.slice(0, sample)
    t = time.time()
    xy = calc_xtx_xty_cpu(params, [sub], min_energy=get_min_energy([data]), n_threads=n_threads)
    dt = time.time() - t
    return xy.total_n_data / dt, dt, xy.total_n_data


NOMINAL_FP32_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12   # 152 SMs x 128 FP32 lanes x FMA at 2,070 MHz
NOMINAL_FP64_TFLOPS = 1.25                            # GB300's FP64 rate (non-tensor)


def eval_flops(model, st, cutoff):
    """Algorithmic flops of one E/F/S evaluation of the structures `st`: per
    neighbour pair (full list) 4 K0(tp) (a_nlm) + 40 K0(tp) (the adjoint's
    pair gradients) + 20 (L+1)^2 (Y_lm and gradients) + 6 G (radial functions),
    and per atom 6 x (feature value and adjoint product terms of its type)."""
    from pypolymlp_gb300 import _ffi

    w = model.work()
    k0 = w["k0_pair"].astype(np.float64)
    ylm = 20.0 * (w["max_l"] + 1) ** 2
    rad = 6.0 * w["n_radial"]
    total = 0.0
    aoff = st.atom_offsets
    for s in range(st.n_st):
        offs, nb, _ = _ffi.neighbor_list(st, s, cutoff)
        t = np.asarray(st.types[aoff[s]:aoff[s + 1]])
        ti = np.repeat(t, np.diff(offs))
        tj = t[nb]
        total += float(np.sum(44.0 * k0[ti, tj]) + len(nb) * (ylm + rad))
        total += 6.0 * float(np.sum(w["n_terms"][t]))
    return total


def eval_bench(params, args):
    """E/F/S atoms/s of the evaluator (pg_eval_run through the C ABI, host
    buffers, neighbour lists included) on bcc cells of n^3 x 2 atoms (a = 3.2 A,
    sigma 0.1 A, 50/50 random species) with the X^T X model, mixed and FP64;
    kernel times from the device profiler; roofline of the mixed evaluator
    against the nominal FP32 CUDA-core peak (no FP32 peak is measured) and of
    the FP64 one against the FP64 rate.  The headline cell is --eval-cell
    (default 20: 16,000 atoms); the 1,024- and 128,000-atom cells of the same
    family are reported beside it (mixed)."""
    import torch

    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300 import synthetic as syn
    from pypolymlp_gb300.abi import Structures

    model = _ffi.Model(params)
    coefs = np.random.default_rng(4).normal(size=model.n_features) * 1e-3
    evs = {_ffi.PG_MIXED: _ffi.Evaluator(params, coefs, _ffi.PG_MIXED),
           _ffi.PG_FP64: _ffi.Evaluator(params, coefs, _ffi.PG_FP64)}

    def cell(n):
        sset = syn.bcc_supercell(n, a=3.2, sigma=0.1, seed=4)
        return Structures(sset.axis, sset.positions, sset.types)

    def one(st, precision, reps=3):
        ev = evs[precision]
        n_atoms = int(st.n_atoms.sum())
        ev.run(st)  # warm-up
        torch.cuda.synchronize()
        _ffi.profile_enable(True)
        _ffi.profile_read()
        t0 = time.time()
        for _ in range(reps):
            ev.run(st)
        dt = (time.time() - t0) / reps
        prof = _ffi.profile_read()
        _ffi.profile_enable(False)
        dev_ms = sum(v[0] for v in prof.values()) / reps
        return {"value": n_atoms / dt, "unit": "atoms/s",
                "device_atoms_per_s": n_atoms / (dev_ms / 1e3) if dev_ms > 0 else None, "device_ms": dev_ms,
                "kernels": {k: {"ms": v[0] / reps, "launches": v[1] // reps} for k, v in prof.items()}}

    st = cell(args.eval_cell)
    n_atoms = int(st.n_atoms.sum())
    mixed = one(st, _ffi.PG_MIXED)
    fp64 = one(st, _ffi.PG_FP64)
    flops = eval_flops(model, st, params["model"]["cutoff"])
    out = {"metric": "E/F/S atoms/s (mixed)", "value": mixed["value"], "unit": "atoms/s",
           "device_atoms_per_s": mixed["device_atoms_per_s"],
           "workload": f"bcc {args.eval_cell}x{args.eval_cell}x{args.eval_cell}x2 = {n_atoms} atoms, a 3.2 A, "
                       f"the X^T X model (F = {len(coefs)})",
           "h2d_bytes": int(st.positions.nbytes + st.axis.nbytes + st.types.nbytes),
           "d2h_bytes": int(n_atoms * 24 + 56), "kernels": mixed["kernels"],
           "fp64": {"value": fp64["value"], "unit": "atoms/s", "device_atoms_per_s": fp64["device_atoms_per_s"],
                    "kernels": fp64["kernels"]},
           "mixed_over_fp64": {"e2e": mixed["value"] / fp64["value"],
                               "device": mixed["device_atoms_per_s"] / fp64["device_atoms_per_s"]}}
    ach32 = flops / (mixed["device_ms"] / 1e3) / 1e12
    ach64 = flops / (fp64["device_ms"] / 1e3) / 1e12
    out["roofline"] = {
        "bound": "fp32 cuda cores", "achieved": ach32, "peak": NOMINAL_FP32_TFLOPS, "unit": "TFLOP/s",
        "frac": ach32 / NOMINAL_FP32_TFLOPS, "flops_per_atom": flops / n_atoms,
        "fp64": {"achieved": ach64, "peak": NOMINAL_FP64_TFLOPS, "frac": ach64 / NOMINAL_FP64_TFLOPS},
        "note": "flops per pair (full list) 44 K0(tp) + 20 (L+1)^2 + 6 G, per atom 6 x product terms of its type; "
                "device time = sum of the evaluation's kernels; peaks nominal (152 SMs x 128 lanes x 2 flops x "
                "2,070 MHz for FP32; 1.25 TFLOP/s FP64)"}
    if not args.no_cpu_baseline:
        # the reference's evaluator restated (oracle, all host threads) on the 1,024-atom cell
        from oracle import oracle

        st8 = cell(8)
        n_threads = os.cpu_count() or 1
        t0 = time.time()
        oracle.evaluate(params, coefs, st8, n_threads=n_threads)
        dt = time.time() - t0
        out["cpu_baseline"] = {"value": 1024 / dt, "unit": "atoms/s", "cores": n_threads, "kind": "port",
                               "sample": f"bcc 8x8x8x2 = 1024 atoms, CPU oracle E/F/S, {dt:.2f}s"}
    out["other_cells"] = {}
    for n in () if args.no_other_cells else (8, 40):
        if n != args.eval_cell:
            r = one(cell(n), _ffi.PG_MIXED)
            out["other_cells"][f"{2 * n ** 3} atoms"] = {"value": r["value"],
                                                         "device_atoms_per_s": r["device_atoms_per_s"]}
    return out


def fit_bench(params, data, args):
    """The full ridge fit of the workload, mixed and FP64: training on the
    first 80 % of the structures, test on the rest, alphas 10^linspace(-3, 1, 5);
    phases timed on the host around the synchronous calls (rows + Gram,
    solve of all alphas, test residual pass); then the energy and force RMSEs
    of both fitted models on the test structures from the FP64 evaluator."""
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.abi import Structures
    from pypolymlp_gb300.accuracy import prediction_errors
    from pypolymlp_gb300.regression import fit

    n = len(data)
    k = int(0.8 * n)
    train, test = data.slice(0, k), data.slice(k, n)
    alphas = [10.0 ** a for a in np.linspace(-3, 1, 5)]
    st = Structures(test.axis, test.positions, test.types)
    offs = np.concatenate([[0], np.cumsum(test.total_n_atoms)])
    out = {"workload": f"{k} training / {n - k} test structures of the X^T X workload", "alphas": alphas}
    for name, prec in (("mixed", _ffi.PG_MIXED), ("fp64", _ffi.PG_FP64)):
        _ffi.profile_enable(True)
        _ffi.profile_read()
        t0 = time.time()
        res = fit(params, [train], [test], alphas, precision=prec)
        wall = time.time() - t0
        prof = _ffi.profile_read()
        _ffi.profile_enable(False)
        ev = _ffi.Evaluator(params, res.scaled_coeffs, _ffi.PG_FP64)
        e, f, s = ev.run(st)
        err, _ = prediction_errors(test, e, [f[offs[i]:offs[i + 1]] for i in range(len(test))], s)
        tm = res.timings
        out[name] = {"seconds": wall, "phases_s": {k2: v for k2, v in tm.items() if k2.endswith("_s")},
                     "xtx_rows_per_s": tm["train_rows"] / tm["assemble_s"], "alpha": res.alpha,
                     "rmse_energy_meV_atom": err["energy"] * 1e3, "rmse_force_meV_A": err["force"] * 1e3,
                     "rmse_test_selected": res.rmse_test,
                     "kernels_ms": {k2: v[0] for k2, v in prof.items()}}
        if "pg_syrk_f64" in prof:
            # the FP64 Gram (the judge path) against the nominal FP64 rate
            F = len(res.scaled_coeffs)
            ach = F * (F + 1) * tm["train_rows"] / (prof["pg_syrk_f64"][0] / 1e3) / 1e12
            out[name]["gram_fp64_roofline"] = {"kernel": "pg_syrk_f64", "bound": "fp64", "achieved": ach,
                                               "peak": 1.25, "unit": "TFLOP/s", "frac": ach / 1.25,
                                               "note": "F(F+1) flops per training row; peak nominal (no FP64 "
                                                       "peak is measured)"}
        log(f"fit {name}: {wall:.1f}s, alpha {res.alpha}, E {err['energy'] * 1e3:.4f} meV/atom, "
            f"F {err['force'] * 1e3:.3f} meV/A")
    m, d = out["mixed"], out["fp64"]
    out["delta_energy_meV_atom"] = abs(m["rmse_energy_meV_atom"] - d["rmse_energy_meV_atom"])
    out["delta_force_meV_A"] = abs(m["rmse_force_meV_A"] - d["rmse_force_meV_A"])
    out["gate"] = bool(out["delta_energy_meV_atom"] < 0.05 and out["delta_force_meV_A"] < 1.0)
    out["fit_speedup_mixed_over_fp64"] = d["seconds"] / m["seconds"]
    out["xtx_speedup_mixed_over_fp64"] = m["xtx_rows_per_s"] / d["xtx_rows_per_s"]
    return out


def cfg5_bench(args):
    """One pass (rows + Gram, mixed) over --cfg5-struct structures of the
    order-4 ternary model (F = 21,945; random triclinic cells of 32-192
    atoms), after one warm-up pass; then the ridge solve of one alpha at that
    size (pg_solve_ridge on the pass's Gram plus its mean diagonal, so that it
    is positive definite)."""
    import torch

    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.params import make_params_dict
    from pypolymlp_gb300.regression import DeviceBatch, GramAccumulator, get_min_energy, solver_ridge

    kw, kind, _, workload = MODELS["cfg5"]
    params = make_params_dict(**kw)
    data = make_dataset(args.cfg5_struct, seed=7, device="cuda", kind=kind, rc=kw["cutoff"])
    model = _ffi.Model(params)
    F = model.n_features
    batch = DeviceBatch(model, data, get_min_energy([data]), _ffi.PG_MIXED)
    gram = GramAccumulator(model, _ffi.PG_MIXED)
    gram.accumulate_batch(batch)  # warm-up (and a first Gram)
    torch.cuda.synchronize()
    _ffi.profile_enable(True)
    _ffi.profile_read()
    gram.reset()
    t0 = time.time()
    gram.accumulate_batch(batch)
    torch.cuda.synchronize()
    dt = time.time() - t0
    prof = _ffi.profile_read()
    _ffi.profile_enable(False)
    xtx, xty, *_ = gram.result()
    gms = prof.get("pg_gram_tc", (0.0, 1))[0]
    g_ach = F * (F + 1) * batch.n_rows / (gms / 1e3) / 1e12 if gms > 0 else None
    _, bf16_tf, peak_kind = measured_peaks()
    sc = np.sqrt(np.maximum(np.diag(xtx), 1e-300))
    A = xtx / np.outer(sc, sc)
    t0 = time.time()
    coefs, info = solver_ridge(A, xty / sc, [1e-3])
    solve_s = time.time() - t0
    solve_tf = (F ** 3 / 3.0 + 2.0 * F * F) / solve_s / 1e12
    return {"workload": workload.replace("50000 structures", f"{len(data)} structures") + f", F = {F}",
            "rows": int(batch.n_rows), "rows_per_s": batch.n_rows / dt, "seconds": dt,
            "gram": {"ms": gms, "achieved": g_ach, "unit": "TFLOP/s", "peak": bf16_tf / 13.0,
                     "frac": g_ach / (bf16_tf / 13.0) if g_ach else None,
                     "note": f"F(F+1) flops per X row; peak = {peak_kind} bf16 dense / 13 (slice products)"},
            "kernels": {k2: {"ms": v[0], "launches": v[1]} for k2, v in prof.items()},
            "solve": {"n_features": F, "alphas": 1, "seconds": solve_s, "info": int(info[0]),
                      "achieved": solve_tf, "peak": 1.25, "unit": "TFLOP/s", "frac": solve_tf / 1.25,
                      "note": "Cholesky of the column-scaled Gram + 1e-3 I and two triangular solves, FP64, "
                              "host copies included; F^3/3 + 2F^2 flops against the nominal FP64 rate"}}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from pypolymlp_gb300.params import make_params_dict

    kw, kind, n_default, workload = MODELS[args.model]
    params = make_params_dict(**kw)
    data = make_dataset(max(args.ref_sample, 8), seed=2, device=None, kind=kind, rc=kw["cutoff"])
    n_threads = os.cpu_count() or 1
    for _ in range(args.warmup if args.warmup < 1 else 1):
        cpu_baseline(params, data, min(4, len(data)), n_threads)
    rates, times = [], []
    for _ in range(args.steps):
        r, dt, rows = cpu_baseline(params, data, args.ref_sample, n_threads)
        rates.append(r)
        times.append(dt)
    value = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload, "model": args.model, "sample_structures": args.ref_sample},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": n_threads, "kind": "port",
                         "sample": f"first {args.ref_sample} structures of the {n_default}-structure workload per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-struct", type=int, default=0, help="structures (default: the model's workload size)")
    ap.add_argument("--model", default="cfg2", choices=sorted(MODELS), help="model and workload (default cfg2)")
    ap.add_argument("--cpu-sample", type=int, default=48)
    ap.add_argument("--ref-sample", type=int, default=48)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--fp64", action="store_true", help="time the FP64 reference-precision path instead")
    ap.add_argument("--no-eval", action="store_true", help="skip the E/F/S evaluation figure")
    ap.add_argument("--eval-cell", type=int, default=20, help="bcc repeats n (n^3 x 2 atoms) of the E/F/S cell")
    ap.add_argument("--no-other-cells", action="store_true",
                    help="E/F/S on the headline cell only (not the 1,024- and 128,000-atom cells)")
    ap.add_argument("--no-fit", action="store_true", help="skip the mixed vs FP64 fit figure")
    ap.add_argument("--no-cfg5", action="store_true", help="skip the order-4 ternary (F = 21,945) figure")
    ap.add_argument("--cfg5-struct", type=int, default=5000, help="structures of the order-4 ternary pass")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch

    rank, world, local_rank = dist_env()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        torch.cuda.set_device(local_rank)
    from pypolymlp_gb300 import _ffi
    from pypolymlp_gb300.abi import Structures
    from pypolymlp_gb300.params import make_params_dict
    from pypolymlp_gb300.regression import DeviceBatch, GramAccumulator, get_min_energy, weights_and_targets

    precision = _ffi.PG_FP64 if args.fp64 else _ffi.PG_MIXED
    kw, kind, n_default, workload = MODELS[args.model]
    params = make_params_dict(**kw)
    n_struct = args.n_struct or n_default
    data = make_dataset(n_struct, seed=2 + rank, device="cuda", kind=kind, rc=kw["cutoff"])
    min_e = get_min_energy([data])
    model = _ffi.Model(params)
    F = model.n_features
    t = time.time()
    batch = DeviceBatch(model, data, min_e, precision)
    log(f"staged {len(data)} structures, {batch.n_rows} rows in {time.time() - t:.1f}s")
    gram = GramAccumulator(model, precision)

    def step():
        gram.reset()
        gram.accumulate_batch(batch)

    for _ in range(max(args.warmup, 0)):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist

            dist.barrier()

    barrier()
    torch.cuda.synchronize()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local_rank) as clk:
        start.record()
        for _ in range(args.steps):
            step()
        end.record()
        torch.cuda.synchronize()
    barrier()
    ms = start.elapsed_time(end)
    if world > 1:
        import torch.distributed as dist

        tt = torch.tensor([ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    rows_per_step = batch.n_rows
    value = rows_per_step * args.steps * world / (ms / 1e3)

    # per-kernel profile of one more step (events on the launching stream)
    _ffi.profile_enable(True)
    _ffi.profile_read()
    step()
    prof = _ffi.profile_read()
    _ffi.profile_enable(False)
    # + per batch: prefix scan, energy-row statistics, row weighting, X^T y (not individually timed)
    launches_per_step = sum(v[1] for v in prof.values()) + 4 * prof.get("pg_nb_count", (0, 1))[1]
    # dominant kernel and its roofline.  X-row kernels (neighbours to rows) are
    # accounted per X row as F x 4 B written + F x 4 B read by the Gram (FP64: x 2),
    # HBM-bound; the Gram per X row as F (F + 1) flops on the tensor cores.
    hbm_gbs, bf16_tf, peak_kind = measured_peaks()
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dname, (dms, dn) = dom
    per_launch_s = dms / dn / 1e3
    row_kernels = ("pg_nb_count", "pg_nb_fill", "pg_nb_mirror", "pg_anlm", "pg_features_adjoint", "pg_rows_pairs",
                   "pg_rows", "pg_rows_es")
    xrow_ms = sum(prof[k][0] for k in row_kernels if k in prof)
    tb = 4 if precision == _ffi.PG_MIXED else 8
    if dname.startswith("pg_gram"):
        flops = F * (F + 1) * rows_per_step / dn
        achieved = flops / per_launch_s / 1e12
        peak = bf16_tf / 13.0 if dname == "pg_gram_tc" else None
        roof = {"kernel": dname, "bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak if peak else None, "traffic": None,
                "note": f"F(F+1) flops per X row; peak = {peak_kind} bf16 dense / 13 (thirteen slice products)"}
    else:
        bytes_ = 2 * F * tb * rows_per_step / dn
        achieved = bytes_ / per_launch_s / 1e9
        sub = 2 * F * tb * rows_per_step / (xrow_ms / 1e3) / 1e9
        traffic = None
        if dname == "pg_rows_pairs" and precision == _ffi.PG_MIXED and args.model in NCU_ROWS_PAIRS_BYTES_PER_ROW:
            traffic = NCU_ROWS_PAIRS_BYTES_PER_ROW[args.model] * rows_per_step / dn / 1e9
        roof = {"kernel": dname, "bound": "hbm", "achieved": achieved, "peak": hbm_gbs, "unit": "GB/s",
                "frac": achieved / hbm_gbs, "traffic": traffic, "traffic_unit": "GB per launch",
                "xrow_subpath": {"kernels": [k for k in row_kernels if k in prof], "ms_per_step": xrow_ms,
                                 "achieved": sub, "frac": sub / hbm_gbs},
                "note": f"algorithmic bytes = F x {tb} B written + F x {tb} B read per X row (the X tile); "
                        f"peak {peak_kind} copy bandwidth; traffic = ncu DRAM bytes per X row of the kernel "
                        f"(one ncu capture of 20 structures) x rows per launch"}
    if "pg_rows_pairs" in prof and precision == _ffi.PG_MIXED:
        # stage A against the FP32 CUDA cores: per neighbour pair of a force
        # structure, 16 flops per adjoint entry of its type pair (T and S_x,y,z:
        # four complex-real products) and 30 per linear feature with entries
        # (the chain rule f S + f' d/r T and the self/virial sums)
        xw = model.xrow_work()
        pc = batch.pair_counts(model.work()["n_type"]).astype(np.float64)
        a_flops = float(np.sum(pc * (16.0 * xw["n_entries"] + 30.0 * xw["n_positions"])))
        ams, an = prof["pg_rows_pairs"]
        a_ach = a_flops / (ams / 1e3) / 1e12
        fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
        roof.setdefault("stage_a_fp32", {
            "kernel": "pg_rows_pairs", "bound": "fp32 cuda cores", "achieved": a_ach, "peak": fp32_peak,
            "unit": "TFLOP/s", "frac": a_ach / fp32_peak, "pairs_per_step": int(pc.sum()),
            "flops_per_step": a_flops,
            "note": "16 flops per (adjoint entry, pair) + 30 per (linear feature with entries, pair), entries of "
                    "the pair's type pair; peak nominal (152 SMs x 128 lanes x 2 flops x 2,070 MHz; no FP32 "
                    "peak is measured)"})
    if "pg_nb_count" in prof and "pg_nb_fill" in prof:
        # the neighbour search against HBM, SURVEY's per-atom bytes: 28 per list
        # entry (int32 neighbour + 3 x FP64 displacement) + 36 per atom
        npairs = int(batch.pair_counts(model.work()["n_type"]).sum())
        n_at = int(sum(data.total_n_atoms))
        nb_s = (prof["pg_nb_count"][0] + prof["pg_nb_fill"][0]) / 1e3
        nb_gbs = (28.0 * npairs + 36.0 * n_at) / nb_s / 1e9
        roof["neighbours"] = {"kernels": ["pg_nb_count", "pg_nb_fill"], "bound": "hbm", "achieved": nb_gbs,
                              "peak": hbm_gbs, "unit": "GB/s", "frac": nb_gbs / hbm_gbs,
                              "note": "28 B per list entry + 36 B per atom; the search itself (candidates x "
                                      "translations per atom) is compute, so the fraction is low"}
    if "pg_gram_tc" in prof and not dname.startswith("pg_gram"):
        gms, gn = prof["pg_gram_tc"]
        g_ach = F * (F + 1) * rows_per_step / (gms / 1e3) / 1e12
        nt = (F + 127) // 128
        tensor_tf = 13 * 2 * 128 * 128 * nt * (nt + 1) / 2 * rows_per_step / (gms / 1e3) / 1e12
        roof["gram"] = {"kernel": "pg_gram_tc", "bound": "tensor", "achieved": g_ach, "peak": bf16_tf / 13.0,
                        "unit": "TFLOP/s", "frac": g_ach / (bf16_tf / 13.0),
                        "tensor_pipe": {"achieved": tensor_tf, "peak": bf16_tf, "frac": tensor_tf / bf16_tf},
                        "note": f"F(F+1) flops per X row; peak = {peak_kind} bf16 dense / 13 (thirteen slice "
                                f"products); tensor_pipe = the 13 BF16 products of every upper 128 x 128 tile "
                                f"over the rows against the bf16 peak"}
    kernels = {k: {"ms_per_step": v[0], "launches": v[1]} for k, v in prof.items()}

    # e2e through the C ABI with host buffers (one pass; host prep + H2D + D2H inside)
    e_row, f_row, s_row, n_rows, w, y = weights_and_targets(data, min_e)
    st = Structures(data.axis, data.positions, data.types)
    gram2 = GramAccumulator(model, precision)
    torch.cuda.synchronize()
    e2e_steps = max(1, min(args.steps, 2))
    t0 = time.time()
    for _ in range(e2e_steps):
        gram2.reset()
        gram2.accumulate(st, e_row, f_row, s_row, n_rows, w, y)
        res = gram2.result()
    torch.cuda.synchronize()
    e2e_s = (time.time() - t0) / e2e_steps
    h2d = st.positions.nbytes + st.axis.nbytes + st.types.nbytes + st.n_atoms.nbytes + 2 * n_rows * 8
    d2h = F * F * 8 + 3 * F * 8
    e2e = {"value": n_rows * world / e2e_s, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(d2h)}
    del res

    ev = eval_bench(params, args) if not args.no_eval and args.model == "cfg2" else None
    fit_obj = fit_bench(params, data, args) if rank == 0 and not args.no_fit and args.model == "cfg2" else None
    cfg5 = cfg5_bench(args) if rank == 0 and not args.no_cfg5 and args.model == "cfg2" else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        n_threads = os.cpu_count() or 1
        r, dt, rows = cpu_baseline(params, data, args.cpu_sample, n_threads)
        cpu = {"value": r, "unit": UNIT, "cores": n_threads, "kind": "port",
               "sample": f"first {args.cpu_sample} structures ({rows} rows), CPU oracle X rows + numpy X^T X, "
                         f"{dt:.1f}s"}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if args.fp64 else "f32 rows + bf16 fixed-point slices",
            "data": "synthetic",
            "config": {"workload": workload.replace(f"{n_default} structures", f"{len(data)} structures")
                       if n_struct != n_default else workload, "model": args.model,
                       "n_features": F, "rows_per_step": int(rows_per_step), "n_structures": len(data),
                       "parallelism": "replicas" if world > 1 else "single",
                       "l2": "inputs larger than L2 (X is rows x F x 4 B)"},
            "gpu_launches": int(launches_per_step * args.steps),
            "roofline": roof,
            "kernels": kernels,
            "e2e": e2e,
            "cpu_baseline": cpu,
            "eval": ev,
            "fit": fit_obj,
            "cfg5": cfg5,
            "clocks": clk.summary(),
        }
        print(json.dumps(line), flush=True)
    return 0


if __name__ == "__main__":
    sys.exit(main())
