"""Benchmark: QC/MM AM1 energy + gradient evaluations per second on one GB300.

Workload: the QC/MM water box (65 QC atoms = 21 waters + hydroxide, charge -1, AM1 RHF, in 4000 TIP3P waters,
NBModelABFS 8/12 A), as a batch of B independent frames (seeded Gaussian displacements of 0.02 A, standing in
for molecular-dynamics frames).  One step = one full energy + gradient of every frame from the diagonal guess
(QC/MM potentials, integrals, SCF to 1e-8 on the density, QC and QC/MM gradients).

value  frames / device time per step, inputs resident on the device (CUDA events on the launching stream);
e2e    the same through System.EnergyBatch with the frames in pinned host memory and energies + gradients
       returned to the host (host<->device copies inside the timed region).
The working set per step (~4 MB per frame, >1 GB per batch) is far larger than L2, so no flush is needed.

--impl reference times the CPU restatement of pDynamo's path (oracle/liboracle.so, built from mndo_oracle.c)
on every host core this process may use: a process pool made and warmed once, each worker holding its QC region
and ABFS spline, each timed step a bounded sample of the same frames split evenly over the workers.
"""

import argparse, hashlib, json, os, subprocess, sys, threading, time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np

# ncu DRAM bytes of one k_scf launch on this workload, per method, with the source hash of the kernel build they were
# captured on; roofline.traffic is reported only when the benched build has the same hash.
SCF_TRAFFIC_PROFILE = os.path.join(HERE, "profiles", "k_scf_dram_qcmm_water_box_304frames.txt")
SCF_SOURCES = ("pdynamo_mirror_gb300/csrc/scf.cu", "pdynamo_mirror_gb300/csrc/common.cuh", "pdynamo_mirror_gb300/csrc/tc.cuh",
               "pdynamo_mirror_gb300/csrc/multipole.cuh", "include/pdg.h")

METRIC = "QC/MM E+grad evals/s at |dE|<1e-6 Eh (AM1 RHF, 65 QC atoms in 4000 TIP3P waters, ABFS 8/12 A)"
UNIT = "evals/s"
KJ = 2625.5


def scf_build_id():
    """Hash of the sources of the SCF kernel's translation unit (what an ncu capture of it describes)."""
    h = hashlib.sha256()
    for rel in SCF_SOURCES:
        with open(os.path.join(HERE, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


def scf_traffic(method, frames):
    """(bytes, note): ncu dram__bytes_read.sum + dram__bytes_write.sum of one k_scf launch of `method` on `frames`
    frames, from the profile summary, when it was captured on this build; (None, why) otherwise."""
    try:
        rec = {}
        with open(SCF_TRAFFIC_PROFILE) as f:
            for line in f:
                if line.strip() and not line.startswith("#"):
                    k, v = line.split(None, 1)
                    rec[k] = v.strip()
    except OSError:
        return None, "no ncu DRAM capture of k_scf"
    if rec.get("build") != scf_build_id():
        return None, "the ncu DRAM capture of k_scf (build %s) is of another build than this one (%s)" % (rec.get("build"), scf_build_id())
    if int(rec.get("frames", 0)) != frames or method + "_dram_read_bytes" not in rec:
        return None, "no ncu DRAM capture of k_scf for this method and batch size"
    return (float(rec[method + "_dram_read_bytes"]) + float(rec[method + "_dram_write_bytes"]),
            "ncu dram__bytes_read.sum + dram__bytes_write.sum of one launch, this build (%s)" % rec["build"])


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except Exception:
        return {}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index=0):
        self.index, self.samples, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.samples.append(parts)

    def stop(self):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[2 + k].lower().startswith("active")})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None, "reasons": reasons}


def fp64_peak_tflops(dev, n=4096, reps=3):
    """cuBLAS DGEMM throughput (torch.matmul, float64, n^3), best of reps: the FP64 roofline peak."""
    import torch
    a = torch.randn(n, n, dtype=torch.float64, device=dev)
    b = torch.randn(n, n, dtype=torch.float64, device=dev)
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e30
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(); torch.matmul(a, b); e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def fp32_peak_tflops(dev, n=4096, reps=3):
    """cuBLAS SGEMM throughput on the CUDA cores (TF32 off), best of reps: the FP32 peak of the mixed method's
    FP32 products."""
    import torch
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        a = torch.randn(n, n, dtype=torch.float32, device=dev)
        b = torch.randn(n, n, dtype=torch.float32, device=dev)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e30
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(); torch.matmul(a, b); e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
    finally:
        torch.backends.cuda.matmul.allow_tf32 = old
    return 2.0 * n ** 3 / (best * 1e-3) / 1e12


def scf_work(T, N, kv, frames, mixed):
    """Algorithmic work of one k_scf launch (all frames) by unit, from the per-frame phase counts:
    FP64 density steps (4/3) N^3 + 3 N^2 kv flops each; the plain method's DIIS saves after FP64 steps 4 N^2 kv,
    its other saves 2 N^3.  Mixed method: FP32 flops of the perturbative base (the back-transformation of the
    nc = N - kv complementary vectors, 2 N^2 nc per FP64 step), of the perturbative steps (the coupling blocks, the
    fixed-point sweeps, the new density), of its FP32 commutators (after FP64 and perturbative steps the factored
    form 4 N^2 kv; after purification steps 2 N^3), and the split-BF16 SP2 products on the tensor cores (6 x 2 N^3
    per SP2 iteration).  Returns flops (fp64, fp32, tensor)."""
    nc = N - kv
    fs = T["QC Densities Steps"].mean()
    cyc = T["QC SCF Fock Builds"].mean()
    if not mixed:
        saves_z = max(fs - 1.0, 0.0)
        f64 = fs * ((4.0 / 3.0) * N ** 3 + 3.0 * N * N * kv) + saves_z * 4.0 * N * N * kv + max(cyc - saves_z, 0.0) * 2.0 * N ** 3
        return frames * f64, 0.0, 0.0
    ps, sw = T["QC Densities Perturbative Steps"].mean(), T["QC Densities Perturbative Sweeps"].mean()
    pur, sp2 = T["QC Densities Purification Steps"].mean(), T["QC Densities SP2 Iterations"].mean()
    f64 = fs * ((4.0 / 3.0) * N ** 3 + 3.0 * N * N * kv)
    pert_fma = (N * N * kv + nc * N * kv + kv * N * kv + N * N * nc + nc * N * nc + kv * nc * N + kv * nc * kv + kv ** 3
                + 2 * kv * kv * N + N * N * kv)
    sweep_fma = kv * nc * kv + nc * (nc + kv) * kv
    f32 = (ps * 2.0 * pert_fma + sw * 2.0 * sweep_fma + (fs + ps) * 4.0 * N * N * kv + fs * 2.0 * N * N * nc
           + pur * 2.0 * N ** 3)
    tc = sp2 * 6 * 2.0 * N ** 3
    return frames * f64, frames * f32, frames * tc


def scf_cta_layout(eng, T):
    """Threads and shared memory of one SCF CTA, and how many CTAs (frames) the SMs actually ran at once,
    from the SM id and %globaltimer interval that every CTA records (pdg_scf_timings)."""
    threads, smem, _ = eng.occupancy()
    sm, st, en = T["SM"].astype(int), T["Start ns"], T["End ns"]
    most = 0
    for s_ in set(sm.tolist()):
        iv = sorted(zip(st[sm == s_], en[sm == s_]))
        for k, (a, b) in enumerate(iv):
            most = max(most, sum(1 for (c, d) in iv if c < b and d > a))
    return {"threads": threads, "shared_bytes": smem, "ctas_per_sm_observed": most, "sms_used": len(set(sm.tolist()))}


def workload(n_frames, seed=1):
    from pdynamo_mirror_gb300 import workloads
    return workloads.qcmm_water_box_frames(n_frames, seed=seed)


def host_cores():
    """Host cores this process may run on."""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ---- CPU baseline: the oracle (the plain-C restatement of the reference's path), one frame after another per process
_CPU = {}


def _cpu_init(Z, Q, sel, charge):
    """Per-process state, made once: the oracle library, the QC region and the ABFS spline knots."""
    sys.path.insert(0, HERE)
    from oracle import oracle as O
    nq = len(sel)
    Zq = [int(z) for z in Z[:nq]]
    _CPU.update(O=O, nq=nq, Q=np.asarray(Q, dtype=np.float64), knots=O.abfs_knots(8.0, 12.0),
                sys=O.System(O.Hamiltonian("am1", Zq), Zq, charge=charge))


def _cpu_frames(frames):
    """Cold energy + gradient of each frame as System.Energy(doGradients=True) computes it: QC/MM potentials, the
    SCF from the diagonal guess, QC gradients, QC/MM gradients.  Returns (frames done, seconds)."""
    O, nq, Q, kn, s = _CPU["O"], _CPU["nq"], _CPU["Q"], _CPU["knots"], _CPU["sys"]
    t0 = time.perf_counter()
    for X in frames:
        phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=kn)
        s.density = None
        r = s.energy(X[:nq], phi=phi)
        O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=kn)
    return len(frames), time.perf_counter() - t0


class CPUBaseline:
    """The oracle on `processes` host cores: a spawned pool made and warmed once (or this process for one core)."""

    def __init__(self, Z, Q, sel, charge, processes):
        self.processes = processes
        self.pool = None
        init = (list(Z), np.asarray(Q), list(sel), int(charge))
        if processes > 1:
            import multiprocessing as mp
            self.pool = mp.get_context("spawn").Pool(processes, initializer=_cpu_init, initargs=init)
        else:
            _cpu_init(*init)

    def warm(self, frames):
        """One frame per worker, outside any timed region."""
        self.run(np.repeat(np.asarray(frames)[:1], self.processes, axis=0))

    def run(self, frames):
        """(wall seconds, frames done, per-worker seconds) for the frames split evenly over the workers."""
        t0 = time.perf_counter()
        if self.pool is None:
            done = [_cpu_frames(frames)]
        else:
            chunks = [c for c in np.array_split(np.asarray(frames), self.processes) if len(c)]
            done = self.pool.map(_cpu_frames, chunks, chunksize=1)
        return time.perf_counter() - t0, sum(d[0] for d in done), [d[1] for d in done]

    def close(self):
        if self.pool is not None:
            self.pool.close()
            self.pool.join()


def run_reference(args):
    Z, X, Q, sel, charge, frames = workload(args.reference_sample)
    cores = host_cores()
    cpu = CPUBaseline(Z, Q, sel, charge, cores)
    cpu.warm(frames)
    times, worker_rates = [], []
    for s in range(args.warmup + args.steps):
        t, n, per = cpu.run(frames)
        if s >= args.warmup:
            times.append(t)
            worker_rates.append(n / max(1, len(per)) / (sum(per) / len(per)))
    cpu.close()
    n = len(frames)
    value = n / (sum(times) / len(times))
    per_core = float(np.mean(worker_rates))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded water box, perturbed frames)",
            "config": {"workload": "qcmm_water_box_am1_abfs", "qc_atoms": len(sel), "mm_atoms": len(Z) - len(sel),
                       "frames_per_step": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "per_core": per_core,
                             "sample": "%d frames per step split evenly over %d worker processes (pool made and warmed once, "
                                       "each worker holding its QC region and spline), cold E+grad per frame, oracle/mndo_oracle.c; "
                                       "per_core = a worker's own frames / its own time, all workers busy" % (n, cores)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


CLUSTER_METRIC = "PM3 E+grad evals/s (512 water clusters of 4-64 molecules, one persistent graph-captured launch)"


def bench_clusters(args):
    """512 independent PM3 water clusters of seeded uniform size 4-64 molecules (N = 24-384) per step, computed
    by MoleculeBatch as one CUDA graph (integrals, the persistent largest-first SCF, gradients), after the
    autotuner picked the SCF schedule.  `value` is the mixed method (split-BF16 purification where N <= 144, FP64
    elsewhere and to convergence); plain FP64 and the per-cluster differences between the two are reported."""
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, MoleculeBatch, workloads, _native
    dev = torch.device("cuda")
    mols = workloads.water_clusters(512, seed=2)
    b = MoleculeBatch("pm3", mols)
    xyz = b.coordinates(mols)
    from pdynamo_mirror_gb300.converger import MIXED_METHOD
    convs = {"fp64": DIISSCFConverger(), "mixed": DIISSCFConverger(**MIXED_METHOD)}
    res = {}
    for name in ("fp64", "mixed"):
        conv = convs[name]
        times = b.autotune(xyz, conv, repeats=1)
        g = b.capture(xyz, conv)
        st = torch.cuda.current_stream()
        for _ in range(args.warmup):
            out = g.launch()
        torch.cuda.synchronize()
        if (out["status"] != 0).any():
            raise SystemExit("%s: SCF did not converge for %d clusters" % (name, int((out["status"] != 0).sum())))
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if name == "mixed" else None
        if clocks:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(args.steps):
            g.launch()
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        clk = clocks.stop() if clocks else None
        T = b.timings()
        # e2e through MoleculeBatch.run: coordinates from pinned host memory, energies + gradients to the host
        host = xyz.cpu().pin_memory()
        te = []
        for k in range(1 + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = b.run(host.to(dev, non_blocking=True), conv)
            E_h, G_h = r["energies"].cpu(), r["gradients"].cpu()
            if k >= 1:
                te.append(time.perf_counter() - t0)
        res[name] = dict(ms=ms, clk=clk, T=T, e2e_s=sum(te) / len(te), E=E_h.numpy(), G=G_h.numpy(),
                         ncyc=out["ncycles"].cpu().numpy(), tuning=b.tuning, h2d=host.numel() * 8,
                         d2h=E_h.numel() * 8 + G_h.numel() * 8)
    head, plain = res["mixed"], res["fp64"]
    n = b.n
    N = np.array(b.n_basis, dtype=np.float64)
    kv = np.array([min(e.n_occupied, e.n_basis - e.n_occupied) for e in b.items], dtype=np.float64)
    T = head["T"]
    fs, ps = T["QC Densities Steps"], T["QC Densities Purification Steps"]
    saves = np.maximum(fs - 1.0, 0.0)
    flops = float(np.sum(fs * ((4.0 / 3.0) * N ** 3 + 3.0 * N * N * kv) + saves * 4.0 * N * N * kv))
    span_ms = (T["End ns"].max() - T["Start ns"].min()) * 1e-6
    fp64_peak = fp64_peak_tflops(dev)
    achieved = flops / (span_ms * 1e-3) / 1e12
    dE = float(np.abs(head["E"][:, 0] - plain["E"][:, 0]).max())
    dG = float(np.abs(head["G"] - plain["G"]).max())
    big = int(np.argmax(N))
    line = {"metric": CLUSTER_METRIC, "value": n / (head["ms"] * 1e-3), "unit": "evals/s", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded water clusters)",
            "config": {"workload": "water_clusters_pm3", "clusters": n, "waters": [4, 64], "basis_functions_mean": float(N.mean()),
                       "basis_functions_max": int(N.max()), "sum_N3": float((N ** 3).sum()), "method": "mixed (purification where N <= 144)",
                       "tensor_items": b.info()["tensor_items"], "autotune": head["tuning"],
                       "mean_scf_cycles": float(head["ncyc"].mean()), "purification_steps_mean": float(ps.mean()),
                       "fp64_density_steps_mean": float(fs.mean()),
                       "largest_cluster_ms": float((T["End ns"][big] - T["Start ns"][big]) * 1e-6), "scf_span_ms": span_ms,
                       "l2": "working set > L2 (no flush needed)"},
            "e2e": {"value": n / head["e2e_s"], "unit": "evals/s", "h2d_bytes_per_step": int(head["h2d"]), "d2h_bytes_per_step": int(head["d2h"])},
            "gpu_launches": 7 * args.steps,
            "roofline": {"bound": "fp64", "kernel": "k_scf_batch", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak, "traffic": None,
                         "note": "algorithmic FP64 flops of the SCF over its span (first CTA start to last CTA end, %%globaltimer); "
                                 "peak = cuBLAS DGEMM 4096^3 in this run (of measured)"},
            "clocks": head["clk"],
            "plain_fp64": {"value": n / (plain["ms"] * 1e-3), "ms_per_step": plain["ms"], "e2e": n / plain["e2e_s"],
                           "mean_scf_cycles": float(plain["ncyc"].mean()), "autotune": plain["tuning"]},
            "accuracy_vs_plain_fp64": {"max_abs_dE_hartree": dE, "max_abs_dF_hartree_per_bohr": dG,
                                       "gate": "|dE| < 1e-6 Eh, |dF| < 1e-5 Eh/Bohr", "pass": bool(dE < 1e-6 and dG < 1e-5)}}
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        order = np.argsort(N)
        sample = order[::32]
        t0 = time.perf_counter()
        for k in sample:
            Zk, Xk = mols[k]
            O.System(O.Hamiltonian("pm3", list(Zk)), list(Zk)).energy(Xk)
        t = time.perf_counter() - t0
        line["cpu_baseline"] = {"value": len(sample) / t * 1.0, "unit": "evals/s", "cores": 1, "kind": "port",
                                "sample": "%d clusters (every 32nd by size, N %d-%d), serial, oracle/mndo_oracle.c; the sample's "
                                          "size mix matches the batch's" % (len(sample), int(N[sample].min()), int(N[sample].max()))}
    print(json.dumps(line))


MD_METRIC = "QC/MM E+grad evals/s in 300 K Langevin dynamics (AM1, 65 QC atoms in 4000 fixed TIP3P waters, ABFS 8/12 A, 0.5 fs)"


def bench_md(args):
    """Config 3 of the metric's workload family: Langevin dynamics (300 K, 0.5 fs, 25 ps^-1) of `frames` replicas
    of the QC/MM water box with the MM waters fixed, every step one energy + gradient per replica.  The learned
    start density is trained on densities converged along training trajectories (seed apart), then evaluated on
    held-out trajectories: (a) cold, against the diagonal guess, on held-out frames; (b) in dynamics, as a
    correction of the extrapolated start (2 P(t-1) - P(t-2) + M(t) - 2 M(t-1) + M(t-2)), against the previous-step
    start (the reference's behaviour) and the plain extrapolation.  The timed comparison: the learned+mixed method
    (its start density kept only where held-out steps show it saves cycles, else the extrapolation) against plain
    FP64 with the previous-step start, each over `steps` dynamics steps after `warmup`, from the same state."""
    import torch
    from pdynamo_mirror_gb300 import (DIISSCFConverger, LangevinDynamics, LearnedDensityGuess, NBModelABFS, QCModelMNDO, System,
                                      workloads)
    rank = int(os.environ.get("RANK", "0"))
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=1)
    R = args.frames
    from pdynamo_mirror_gb300.converger import MIXED_METHOD as MIXED

    def make(method):
        s = System(Z, X, mmCharges=Q)
        s.electronicState.charge = charge
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**(MIXED if method == "mixed" else {}))), qcSelection=sel)
        s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
        s.DefineFixedAtoms(range(len(sel), len(Z)))
        return s

    def equilibrate(m):
        """The seeded start geometry is not relaxed: a strongly damped bath (250 ps^-1) carries off the released
        energy, then the production bath (25 ps^-1) for a third of the steps."""
        m.set_bath(collisionFrequency=250.0)
        m.run(args.md_equilibration)
        m.set_bath(collisionFrequency=25.0)
        m.run(args.md_equilibration // 3)

    info = {}
    t0 = time.perf_counter()
    s_tr = make("fp64")
    md = LangevinDynamics(s_tr, replicas=R, timeStep=0.0005, seed=101 + rank, densityGuess="extrapolate")
    equilibrate(md)
    frames, phis, dens = [], [], []

    def keep(m, r):
        frames.append(m.xyz.clone()); phis.append(r["phi"].clone()); dens.append(m.history[-1].clone())
    md.run(args.md_training_steps, keep)
    Ft, PHt, Pt = torch.cat(frames), torch.cat(phis), torch.cat(dens)
    del frames, phis, dens
    g = LearnedDensityGuess(s_tr.engine(), seed=0)
    hist = g.fit(Ft, PHt, Pt, epochs=args.md_epochs, batch=64, lr=1e-3, seed=0)
    hist += g.fit(Ft, PHt, Pt, epochs=max(1, args.md_epochs // 2), batch=64, lr=2e-4, seed=1)
    torch.cuda.synchronize()
    info.update(training_densities=int(Ft.shape[0]), training_trajectories=R, training_seconds=time.perf_counter() - t0,
                loss_first_last=[hist[0], hist[-1]])
    del Ft, PHt, Pt
    # held-out trajectories: equilibrate, then snapshot the state every method starts from
    s_ho = make("fp64")
    ho = LangevinDynamics(s_ho, replicas=R, timeStep=0.0005, seed=202 + rank, densityGuess="extrapolate")
    equilibrate(ho)
    snap = dict(X=ho.X.clone(), vel=ho.vel.clone(), acc=ho.acc.clone(), hist=[h.clone() for h in ho.history], n=ho.n_step)
    # (a) cold start on held-out frames: learned guess against the diagonal guess
    cold = LearnedDensityGuess(s_ho.engine(), seed=0)
    cold.load_state_dict(g.state_dict())
    info["cold_start"] = cold.validate(ho.xyz.contiguous(), s_ho.qcModel.converger, ho.mm_xyz, ho.mm_q, s_ho.nbModel)

    def run_mode(method, mode, steps, warm, clocks=None):
        s = make(method)
        guess = mode
        if mode == "learned":
            guess = LearnedDensityGuess(s.engine(), seed=0)
            guess.load_state_dict(g.state_dict())
        m = LangevinDynamics(s, replicas=R, timeStep=0.0005, seed=202 + rank, densityGuess=guess)
        m.X.copy_(snap["X"]); m.vel.copy_(snap["vel"]); m.acc.copy_(snap["acc"]); m.n_step = snap["n"]
        m.history = [h.clone() for h in snap["hist"]]
        m.last = {}
        m.run(warm)
        torch.cuda.synchronize()
        st = torch.cuda.current_stream()
        if clocks:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        cyc = m.run(steps)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        clk = clocks.stop() if clocks else None
        E = m.last["energies"][:, 0].cpu().numpy()
        G = (m.last["qc_gradients"] + m.last["qcmm_qc_gradients"]).cpu().numpy()
        T = m.temperatures()[1]
        return dict(ms=ms, evals=R / (ms * 1e-3), cycles=float(np.mean([c.double().mean().item() for c in cyc])), E=E, G=G,
                    T=float(T.mean()), clk=clk, xyz=m.xyz.clone(), md=m)

    modes = {}
    for method, mode in (("fp64", "previous"), ("fp64", "extrapolate"), ("fp64", "learned"), ("mixed", "previous"),
                         ("mixed", "extrapolate"), ("mixed", "learned")):
        modes[(method, mode)] = run_mode(method, mode, args.md_compare_steps, 3)
    # the learned correction is kept only if it makes the held-out steps faster (cycles saved net of its inference)
    use_learned = modes[("mixed", "learned")]["evals"] > modes[("mixed", "extrapolate")]["evals"]
    best = "learned" if use_learned else "extrapolate"
    # timed: learned+mixed (as validated) against plain FP64 with the reference's previous-step start
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    head = run_mode("mixed", best, args.steps, args.warmup, clocks)
    plain = run_mode("fp64", "previous", args.steps, args.warmup)
    # accuracy: plain FP64 (cold, diagonal guess) on the last geometry of the timed learned+mixed trajectories
    hm = head["md"]
    ref = make("fp64")
    r = ref.engine().run(head["xyz"], ref.qcModel.converger, hm.mm_xyz, hm.mm_q, ref.nbModel, gradients=True, warm_start=False,
                         mm_gradients=False)
    dE = float(np.abs(head["E"] - r["energies"][:, 0].cpu().numpy()).max())
    dG = float(np.abs(head["G"] - (r["qc_gradients"] + r["qcmm_qc_gradients"]).cpu().numpy()).max())
    del head["md"], plain["md"]
    line = {"metric": MD_METRIC, "value": head["evals"], "unit": UNIT, "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water box; Langevin trajectories of its QC atoms)",
            "config": {"workload": "qcmm_water_box_langevin", "replicas": R, "time_step_fs": 0.5, "temperature_k": 300.0,
                       "collision_frequency_per_ps": 25.0,
                       "equilibration": "%d steps at 250 ps^-1, %d at 25 ps^-1" % (args.md_equilibration, args.md_equilibration // 3),
                       "method": "learned+mixed: mixed density steps, start density %s" % (
                           "extrapolation + learned correction" if use_learned else "extrapolation (the learned correction did not make held-out steps faster)"),
                       "mean_scf_cycles": head["cycles"], "mean_temperature_k": head["T"],
                       "l2": "working set > L2 (no flush needed)"},
            # per step: positions, QC/MM potentials, 4 integral kernels, SCF, 4 gradient kernels, 2 QC/MM gradient
            # kernels, velocities, and the start-density combination; the learned correction adds its features (4),
            # three MLP layers, the assembly and a potentials launch
            "gpu_launches": (16 + (9 if use_learned else 0)) * args.steps,
            "clocks": head["clk"],
            "plain_fp64_previous_start": {"value": plain["evals"], "ms_per_step": plain["ms"], "mean_scf_cycles": plain["cycles"]},
            "start_density_comparison": {"%s/%s" % k: {"evals_per_s": v["evals"], "mean_scf_cycles": v["cycles"]} for k, v in modes.items()},
            "learned_guess": info,
            "accuracy_vs_plain_fp64": {"where": "last geometry of every timed learned+mixed trajectory, plain FP64 from the diagonal guess",
                                       "max_abs_dE_hartree": dE,
                                       "max_abs_dF_hartree_per_bohr": dG, "gate": "|dE| < 1e-6 Eh, |dF| < 1e-5 Eh/Bohr",
                                       "pass": bool(dE < 1e-6 and dG < 1e-5)}}
    print(json.dumps(line))


LARGE_METRIC = ("QC/MM E+grad per MD step, evals/s (AM1, 200 QC waters = 600 atoms, N = 1200, in 20000 fixed TIP3P waters, "
                "ABFS 8/12 A, 300 K Langevin, 0.5 fs)")


def large_cpu_sample(Z, Q, sel, charge, X):
    """The oracle on one host core for the large frame, bounded: integrals + SCF cycles + gradients cost T(c) for c
    SCF cycles; runs with c = 1 and c = 2 give the fixed cost and the cost per cycle (seconds)."""
    from oracle import oracle as O
    nq = len(sel)
    Zq = [int(z) for z in Z[:nq]]
    ham = O.Hamiltonian("am1", Zq)
    kn = O.abfs_knots(8.0, 12.0)
    t = {}
    for c in (1, 2):
        s = O.System(ham, Zq, charge=charge, maximumSCFCycles=c)
        t0 = time.perf_counter()
        phi = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=kn)[0]
        r = s.energy(X[:nq], phi=phi)
        O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=kn)
        t[c] = time.perf_counter() - t0
    per_cycle = t[2] - t[1]
    return t[1] - per_cycle, per_cycle


def bench_large(args, md_steps=None, md_warmup=None, cpu=True):
    """The large QC/MM system: Langevin dynamics (300 K, 0.5 fs, 25 ps^-1) of its 600 QC atoms in the fixed MM waters,
    every step one E+grad with the previous step's density as the start (the reference's warm start), each SCF over the
    whole GPU (the wide engine).  Plain FP64 against the mixed method (FP64 base steps, perturbative steps around the
    base kept across MD steps, FP32 DIIS errors and pair-gradient terms) from the same start; ms per MD step by CUDA
    events over the timed steps.  Accuracy: plain FP64 cold E+grad at the last geometry of the mixed trajectory."""
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, LangevinDynamics, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD
    steps = args.steps if md_steps is None else md_steps
    warm = max(3, args.warmup if md_warmup is None else md_warmup)
    Z, X, Q, sel, charge = workloads.large_qcmm()
    nq = len(sel)

    def make(method):
        s = System(Z, X, mmCharges=Q)
        s.electronicState.charge = charge
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**(MIXED_METHOD if method == "mixed" else {}))), qcSelection=sel)
        s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
        s.DefineFixedAtoms(range(nq, len(Z)))
        return s

    res = {}
    for method in ("fp64", "mixed"):
        s = make(method)
        eng = s.engine()
        eng.wide_phase_events(True)
        md = LangevinDynamics(s, replicas=1, timeStep=0.0005, seed=404, densityGuess="previous")
        t0 = time.perf_counter()
        md.run(1)
        torch.cuda.synchronize()
        cold_ms = 1e3 * (time.perf_counter() - t0)
        md.run(warm - 1)
        torch.cuda.synchronize()
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if method == "mixed" else None
        if clocks:
            clocks.start()
        st = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        phases = []
        e0.record(st)
        cyc = []
        for _ in range(steps):
            cyc += md.run(1)
            phases.append(eng.wide_phase_times())
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        res[method] = dict(ms=ms, cold_ms=cold_ms, clk=clocks.stop() if clocks else None,
                           cycles=float(np.mean([int(c[0]) for c in cyc])),
                           phases={k: float(np.mean([p[k] for p in phases])) for k in phases[0]},
                           E=float(md.last["energies"][0, 0]), G=(md.last["qc_gradients"] + md.last["qcmm_qc_gradients"])[0].cpu().numpy(),
                           xyz=md.xyz.clone(), mm=(md.mm_xyz, md.mm_q), nb=s.nbModel)
    head, plain = res["mixed"], res["fp64"]
    ref = make("fp64")
    r = ref.engine().run(head["xyz"], ref.qcModel.converger, head["mm"][0], head["mm"][1], head["nb"], gradients=True,
                         warm_start=False, mm_gradients=False)
    dE = abs(head["E"] - float(r["energies"][0, 0]))
    dG = float(np.abs(head["G"] - (r["qc_gradients"] + r["qcmm_qc_gradients"])[0].cpu().numpy()).max())
    out = {"metric": LARGE_METRIC, "value": 1e3 / head["ms"], "unit": UNIT, "ms_per_md_step": head["ms"], "md_steps": steps,
           "warmup_md_steps": warm, "higher_is_better": True,
           "config": {"workload": "large_qcmm_am1_abfs_langevin", "qc_atoms": nq, "basis_functions": ref.engine().n_basis,
                      "mm_atoms": len(Z) - nq, "time_step_fs": 0.5, "temperature_k": 300.0, "start_density": "previous step (warm)",
                      "engine": "wide (one frame over all SMs)", "method": "mixed: FP64 base steps + perturbative steps around the "
                      "base kept across MD steps (no purification beyond 144 basis functions; no learned start density)"},
           "mean_scf_cycles": head["cycles"], "cold_first_step_ms": head["cold_ms"], "phase_ms_per_md_step": head["phases"],
           "plain_fp64": {"value": 1e3 / plain["ms"], "ms_per_md_step": plain["ms"], "mean_scf_cycles": plain["cycles"],
                          "cold_first_step_ms": plain["cold_ms"], "phase_ms_per_md_step": plain["phases"]},
           "accuracy_vs_plain_fp64": {"where": "last geometry of the timed mixed trajectory, plain FP64 cold", "max_abs_dE_hartree": dE,
                                      "max_abs_dF_hartree_per_bohr": dG, "gate": "|dE| < 1e-6 Eh, |dF| < 1e-5 Eh/Bohr",
                                      "pass": bool(dE < 1e-6 and dG < 1e-5)},
           "clocks": head["clk"]}
    if cpu:
        fixed, per_cycle = large_cpu_sample(Z, Q, sel, charge, X)
        est = fixed + plain["cycles"] * per_cycle
        out["cpu_baseline"] = {"value": 1.0 / est, "unit": UNIT, "cores": 1, "kind": "port",
                               "sample": "oracle/mndo_oracle.c on the 600-atom frame with 1 and 2 SCF cycles (fixed cost %.1f s, "
                                         "%.1f s per cycle), taken at the plain GPU path's %.2f warm cycles per MD step"
                                         % (fixed, per_cycle, plain["cycles"])}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--frames", type=int, default=304, help="frames per step per GPU")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--reference-sample", type=int, default=256)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--method", default="learned_mixed", choices=["learned_mixed", "mixed", "fp64"],
                    help="learned start density + purification cycles (the metric's learned+mixed), purification cycles "
                         "from the diagonal guess (mixed), or FP64 throughout")
    ap.add_argument("--workload", default="qcmm_water_box", choices=["qcmm_water_box", "water_clusters", "qcmm_md", "large_qcmm"],
                    help="the QC/MM water box (the headline metric), 512 independent PM3 water clusters in one launch, or "
                         "Langevin dynamics of water-box replicas with the learned start density trained on trajectories")
    ap.add_argument("--no-large", action="store_true", help="leave out the large QC/MM sub-line of the default workload")
    ap.add_argument("--profile-region", action="store_true",
                    help="bracket the reported method's timed steps with cudaProfilerStart/Stop (for ncu --profile-from-start off) "
                         "and time only that method")
    ap.add_argument("--large-steps", type=int, default=10, help="timed MD steps per method of the large QC/MM sub-line")
    ap.add_argument("--md-equilibration", type=int, default=150)
    ap.add_argument("--md-training-steps", type=int, default=66, help="training densities = replicas x this")
    ap.add_argument("--md-epochs", type=int, default=6)
    ap.add_argument("--md-compare-steps", type=int, default=12)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.workload == "water_clusters" and args.impl == "gb300":
        return bench_clusters(args)
    if args.workload == "qcmm_md" and args.impl == "gb300":
        return bench_md(args)
    if args.workload == "large_qcmm" and args.impl == "gb300":
        print(json.dumps(bench_large(args, cpu=not args.no_cpu_baseline)))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    bench_water_box(args, world, rank)


def tei_count(Z):
    """Two-centre TEIs of a QC region: per atom pair n_i(n_i+1)/2 x n_j(n_j+1)/2 (4 orbitals on heavy atoms, 1 on H)."""
    t = np.array([1 if int(z) == 1 else 10 for z in Z], dtype=np.int64)
    return int((t.sum() ** 2 - (t * t).sum()) // 2)


def qcmm_pairs_in_cutoff(qc, mm, cutoff):
    """QC/MM pairs within the outer cutoff over all frames (device tensors [F, n, 3], [F, m, 3] in A)."""
    import torch
    n = 0
    for f0 in range(0, qc.shape[0], 16):
        d = torch.cdist(qc[f0:f0 + 16], mm[f0:f0 + 16])
        n += int((d < cutoff).sum().item())
    return n


def single_frame_latency(Z, X, Q, sel, charge, method, repeats=5):
    """Median wall time (ms) of one cold System.EnergyBatch(doGradients=True) of one frame, host coordinates in and
    energy + gradients out: the drop-in call's latency.  method "shared": the mixed method with a shared base taken
    from a first call on another perturbed frame, each timed call on a perturbed frame of its own (sigma 0.02 A)."""
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD, SHARED_BASE_METHOD
    s = System(Z, X, mmCharges=Q if Q is not None else None)
    s.electronicState.charge = charge
    opts = {"mixed": MIXED_METHOD, "shared": SHARED_BASE_METHOD}.get(method, {})
    s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**opts)), qcSelection=sel)
    if Q is not None:
        s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
    frames = workloads.perturbed_frames(X, 2 + repeats, sigma=0.02, seed=77) if method == "shared" else np.repeat(X[None], 2 + repeats, 0)
    t = []
    for k in range(2 + repeats):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.EnergyBatch(frames[k:k + 1], doGradients=True, warmStart=False)
        if k >= 2:
            t.append(time.perf_counter() - t0)
    return 1e3 * float(np.median(t))


def cpu_single_frame(Z, X, Q, sel, charge, repeats=3):
    """Median wall time (ms) of the oracle's cold E+grad of the same frame on one host core."""
    from oracle import oracle as O
    nq = len(sel)
    Zq = [int(z) for z in Z[:nq]]
    s = O.System(O.Hamiltonian("am1", Zq), Zq, charge=charge)
    kn = O.abfs_knots(8.0, 12.0) if Q is not None else None
    t = []
    for _ in range(repeats):
        t0 = time.perf_counter()
        phi = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=kn)[0] if Q is not None else None
        s.density = None
        r = s.energy(X[:nq], phi=phi)
        if Q is not None:
            O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=kn)
        t.append(time.perf_counter() - t0)
    return 1e3 * float(np.median(t))


def bench_water_box(args, world, rank):
    import torch
    from pdynamo_mirror_gb300 import DIISSCFConverger, NBModelABFS, QCModelMNDO, System, _native, workloads
    from pdynamo_mirror_gb300.converger import MIXED_METHOD, SHARED_BASE_METHOD
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda")
    Z, X, Q, sel, charge, frames = workload(args.frames, seed=1 + rank)
    METHODS = {"fp64": dict(densityStep="fp64"), "mixed": dict(MIXED_METHOD), "learned_mixed": dict(SHARED_BASE_METHOD)}
    # a fresh set of perturbed frames for every step (warm-up and timed), the same sets for every method: the shared
    # base of the headline method comes from frames no timed step evaluates
    n_sets = args.warmup + args.steps
    frame_sets = [frames] + [workloads.perturbed_frames(X, args.frames, sigma=0.02, seed=11 + k) for k in range(1, n_sets)]
    guess_info = {}
    nq = len(sel)

    def train_guess(s, eng):
        """The learned start density (LinearResponseGuess), fitted to the densities the SCF converges here on 2048
        frames of their own seed (the first of those batches also leaves the shared base); returns the model."""
        from pdynamo_mirror_gb300 import LinearResponseGuess
        t0 = time.perf_counter()
        tr = workloads.perturbed_frames(X, 2048, sigma=0.02, seed=101 + rank)
        qc_t, mm_t, q_t, _ = s._device_inputs(tr)
        g = LinearResponseGuess(eng)
        for s0 in range(0, len(tr), 256):
            r = eng.run(qc_t[s0:s0 + 256].contiguous(), s.qcModel.converger, mm_t[s0:s0 + 256].contiguous(), q_t, s.nbModel,
                        gradients=False, warm_start=False)
            g.fit(qc_t[s0:s0 + 256], r["phi"], eng.density)
        del qc_t, mm_t
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        return g, {"training_frames": len(tr), "train_seconds": time.perf_counter() - t0}

    def measure(method, timed_clocks):
        s = System(Z, X, mmCharges=Q)
        s.electronicState.charge = charge
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**METHODS[method])), qcSelection=sel)
        s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
        eng = s.engine()
        dev_sets = []
        for fs in frame_sets:
            qc, mm, q, mm_idx = s._device_inputs(fs)
            dev_sets.append((qc, mm))
        conv, nb = s.qcModel.converger, s.nbModel
        # the e2e inputs: every frame set in pinned host memory, allocated and copied to the device once here, before
        # any timing (on this host the first copies out of freshly pinned memory run at a fraction of the link's
        # bandwidth until the driver has mapped the pages; a caller reuses its pinned buffers)
        sets_h = [torch.from_numpy(np.ascontiguousarray(fs)).pin_memory() for fs in frame_sets]
        for fh in sets_h:
            fh.to(dev, non_blocking=True)
        torch.cuda.synchronize()
        guess = None
        if method == "learned_mixed":
            guess, info = train_guess(s, eng)
            s.DefineDensityGuess(guess)
            # held-out validation (frames of their own seed): the guess stays on only if it saves SCF cycles
            qc_v, mm_v, q_v, _ = s._device_inputs(workloads.perturbed_frames(X, 256, sigma=0.02, seed=201 + rank))
            info.update(guess.validate(qc_v, conv, mm_v, q_v, nb))
            info["used_in_timed_steps"] = guess.enabled
            guess_info.update(info)

        def step(k, events=False):
            qc, mm = dev_sets[k % n_sets]
            return eng.run(qc, conv, mm, q, nb, gradients=True, warm_start=False, guess=guess, events=events)

        for k in range(args.warmup):
            r = step(k)
        torch.cuda.synchronize()
        st = r["status"].cpu().numpy()
        if (st != 0).any():
            raise SystemExit("%s: SCF did not converge for %d frames" % (method, int((st != 0).sum())))
        stream = torch.cuda.current_stream()
        clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if timed_clocks else None
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        if clocks:
            clocks.start()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        profiled = args.profile_region and timed_clocks
        if profiled:
            torch.cuda.profiler.start()
        e0.record(stream)
        for k in range(args.steps):
            r = step(args.warmup + k)
        e1.record(stream)
        torch.cuda.synchronize()
        if profiled:
            torch.cuda.profiler.stop()
        if world > 1:
            torch.distributed.barrier()
        ms = e0.elapsed_time(e1) / args.steps
        clk = clocks.stop() if clocks else None
        timers = eng.timings(len(frames))
        # per-phase device times of further steps (not the timed ones): CUDA events around the QC/MM potentials,
        # the integral kernels, the SCF kernel, the gradient kernels and the QC/MM gradients, median of 3
        eng.phase_events(True)
        phases = []
        for k in range(3):
            rr = step(args.warmup + k, events=True)
            torch.cuda.synchronize()
            pt = eng.phase_times()
            ev = rr["events"]
            pt.update(qcmm_potentials=ev[0].elapsed_time(ev[1]), qcmm_gradients=ev[2].elapsed_time(ev[3]),
                      step=ev[0].elapsed_time(ev[3]))
            phases.append(pt)
        eng.phase_events(False)
        phase_ms = {k: float(np.median([p[k] for p in phases])) for k in phases[0]}
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        # e2e through the public API: frames from pinned host memory in, energies and gradients out
        for fh in sets_h:   # one more untimed pass over the pinned inputs
            fh.to(dev, non_blocking=True)
        torch.cuda.synchronize()
        te = []
        e2e_warm = args.warmup + 2   # untimed calls: the host's first copies out of the pinned inputs and the first
                                     # pinned result buffers are slower
        for k in range(e2e_warm + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            E, G, terms = s.EnergyBatch(sets_h[k % n_sets], doGradients=True, warmStart=False)
            torch.cuda.synchronize()
            if k >= e2e_warm:
                te.append(time.perf_counter() - t0)
        qc, mm = dev_sets[0]
        return dict(ms=ms, clk=clk, phase_ms=phase_ms, e2e_s=sum(te) / len(te), e2e_ms_each=[1e3 * t for t in te], E=E, G=G,
                    ncyc=r["ncycles"].cpu().numpy(), timers=timers, eng=eng, conv=conv, frames_h=sets_h[0], qc=qc, mm=mm)

    if args.profile_region:
        # only the reported method, its timed steps inside the profiler range
        h = measure(args.method, True)
        if rank == 0:
            print(json.dumps({"profile_region": args.method, "frames": len(frames), "steps": args.steps, "ms_per_step": h["ms"]}))
        return
    plain = measure("fp64", args.method == "fp64")
    mixed = None if args.method == "fp64" else (measure("mixed", args.method == "mixed"))
    head = plain if args.method == "fp64" else (mixed if args.method == "mixed" else measure(args.method, True))
    eng, conv = head["eng"], head["conv"]
    n_total = len(frames) * world
    value = n_total / (head["ms"] * 1e-3)
    e2e = n_total / head["e2e_s"]
    N, kv = eng.n_basis, min(eng.n_occupied, eng.n_basis - eng.n_occupied)
    T = head["timers"]
    fp64_steps = float(T["QC Densities Steps"].mean())
    pur_steps = float(T["QC Densities Purification Steps"].mean())
    ncyc_f = float(head["ncyc"].mean())
    fp64_peak = fp64_peak_tflops(dev)
    fp32_peak = fp32_peak_tflops(dev)
    pk = peaks()
    bf16_peak = pk.get("bf16_tflops", 1898.3)
    hbm_peak = pk.get("hbm_gbs", 6790.0)
    nF = len(frames)

    def roofline(h, mixed):
        """FP64 roofline of the method's k_scf (its FP64 algorithmic flops over the event-timed launch, against
        cuBLAS DGEMM measured here) and, for the mixed method, the composite: the time its FP64, FP32 and tensor work
        would take at the three measured peaks over the measured time."""
        f64, f32, tc = scf_work(h["timers"], N, kv, nF, mixed)
        t_ms = h["phase_ms"]["scf"]
        t = t_ms * 1e-3
        traffic, tnote = scf_traffic("mixed" if mixed else "fp64", nF)
        # the pipe that bounds the kernel's algorithmic work: FP64 for the plain method; for the mixed method the one
        # whose work takes longest at its measured peak (the FP32 pipe when every step is perturbative)
        unit_work = {"fp64": (f64, fp64_peak, "cuBLAS DGEMM 4096^3 measured in this run (MEASURED_PEAKS.json has no FP64 figure)"),
                     "fp32": (f32, fp32_peak, "cuBLAS SGEMM 4096^3 without TF32, measured in this run"),
                     "tensor": (tc, bf16_peak, "MEASURED_PEAKS.json bf16 burst")}
        bound = "fp64" if not mixed else max(unit_work, key=lambda u: unit_work[u][0] / unit_work[u][1])
        work, peak, pnote = unit_work[bound]
        r = {"bound": bound, "kernel": "k_scf", "achieved": work / t / 1e12, "peak": peak, "unit": "TFLOP/s",
             "frac": work / t / 1e12 / peak, "traffic": traffic, "traffic_note": tnote,
             "dram_throughput_frac": None if traffic is None else traffic / t / 1e9 / hbm_peak,
             "note": "%s algorithmic flops of the k_scf launch (%.2f ms, %d frames, CUDA events on its stream) against %s "
                     "(of measured); dram_throughput_frac = the ncu traffic over the launch against the measured HBM copy "
                     "bandwidth" % (bound.upper(), t_ms, nF, pnote)}
        if mixed:
            t_ideal = f64 / (fp64_peak * 1e12) + f32 / (fp32_peak * 1e12) + tc / (bf16_peak * 1e12)
            r["composite"] = {"t_ideal_ms": t_ideal * 1e3, "t_measured_ms": t_ms, "frac": t_ideal / t,
                              "fp64_tflop": f64 / 1e12, "fp32_tflop": f32 / 1e12, "tensor_tflop": tc / 1e12,
                              "fp32_peak_tflops": fp32_peak, "bf16_peak_tflops": bf16_peak,
                              "note": "the mixed SCF spreads its work over the FP64 pipe (FP64 base steps), the FP32 pipe (perturbative "
                                      "steps, commutators) and the tensor cores (SP2): time at the three measured peaks (FP32: cuBLAS "
                                      "SGEMM 4096^3 without TF32, measured here; BF16 burst: MEASURED_PEAKS.json) over the measured launch"}
        return r

    def kernel_rooflines(h):
        """Roofline of every kernel group of one step against the measured HBM copy bandwidth, from the algorithmic
        bytes per unit of work: integrals 8 (n_TEI + N(N+1)/2 + 20 n_pairs) written + 24 N_A read per frame; Fock
        builds 8 n_TEI + 24 N(N+1)/2 per build (their share of the SCF launch from its per-CTA phase cycles);
        gradients 8 (n_TEI + N(N+1)/2) read + 24 N_A written per frame; QC/MM potentials and gradients 32 bytes per
        QC/MM pair within the outer cutoff."""
        ph, Th = h["phase_ms"], h["timers"]
        n_tei, npk = tei_count(Z[:nq]), N * (N + 1) // 2
        n_pairs = nq * (nq - 1) // 2
        builds = float(Th["QC SCF Fock Builds"].mean())
        fock_share = float(Th["QC Fock"].mean() / Th["QC SCF Total"].mean())
        pairs = qcmm_pairs_in_cutoff(h["qc"], h["mm"], 12.0)

        def row(kernels, nbytes, ms, unit_note):
            gbs = nbytes / (ms * 1e-3) / 1e9
            return {"kernels": kernels, "bound": "hbm", "bytes": nbytes, "ms": ms, "achieved": gbs, "peak": hbm_peak,
                    "unit": "GB/s", "frac": gbs / hbm_peak, "count": unit_note}
        return {
            "pair_integrals": row("k_pair_integrals, _ss, _sps, k_assemble_h", nF * (8 * (n_tei + npk + 20 * n_pairs) + 24 * nq),
                                  ph["integrals"], "n_TEI %d, N %d, %d pairs per frame" % (n_tei, N, n_pairs)),
            "fock_build": row("k_scf (Fock build share %.3f of the launch)" % fock_share, nF * builds * (8 * n_tei + 24 * npk),
                              fock_share * ph["scf"], "%.2f builds per frame" % builds),
            "gradients": row("k_pair_gradients, _ss, _sps, k_reduce_gradients", nF * (8 * (n_tei + npk) + 24 * nq), ph["gradients"],
                             "n_TEI %d per frame" % n_tei),
            "qcmm_potentials": row("k_qcmm_potentials", 32 * pairs, ph["qcmm_potentials"], "%d QC/MM pairs within 12 A" % pairs),
            "qcmm_gradients": row("k_qcmm_grad_qc, k_qcmm_grad_mm (FP32 pair terms in the mixed method)", 32 * pairs,
                                  ph["qcmm_gradients"], "%d QC/MM pairs within 12 A" % pairs),
            "phase_ms": ph,
            "note": "CUDA events on the launching stream around each kernel group of one step (median of 3 steps after the "
                    "timed ones); peak = MEASURED_PEAKS.json hbm_gbs (of measured)"}

    clk = head["clk"]
    # one QC/MM E+grad (the drop-in call) and one 16-water AM1 E+grad: latency through System.EnergyBatch, and the oracle
    # on one host core
    Z0, X0 = workloads.water_cluster(16, seed=0)
    single = {"qcmm_water_box": {"gpu_ms_plain_fp64": single_frame_latency(Z, X, Q, sel, charge, "fp64"),
                                 "gpu_ms_mixed": single_frame_latency(Z, X, Q, sel, charge, "mixed"),
                                 "gpu_ms_mixed_shared_base": single_frame_latency(Z, X, Q, sel, charge, "shared"),
                                 "cpu_ms_one_core": cpu_single_frame(Z, X, Q, sel, charge) if not args.no_cpu_baseline else None},
              "water_cluster_16_am1": {"gpu_ms_plain_fp64": single_frame_latency(Z0, X0, None, list(range(len(Z0))), 0, "fp64"),
                                       "gpu_ms_mixed": single_frame_latency(Z0, X0, None, list(range(len(Z0))), 0, "mixed"),
                                       "cpu_ms_one_core": cpu_single_frame(Z0, X0, None, list(range(len(Z0))), 0) if not args.no_cpu_baseline else None},
              "note": "median wall time of one cold System.EnergyBatch(doGradients=True) of one frame (host coordinates in, energy "
                      "and gradients out; one SCF CTA on one SM), and of the oracle's cold E+grad of the same frame on one host core"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water box, perturbed frames)",
            "config": {"workload": "qcmm_water_box_am1_abfs", "qc_atoms": nq, "mm_atoms": len(Z) - nq,
                       "basis_functions": N, "frames_per_step": nF,
                       "method": {"fp64": "plain FP64",
                                  "mixed": "mixed: split-BF16 SP2 purification on tcgen05 (6 partial products, FP32 accumulation) until the RMS density change < 1e-5, then FP64",
                                  "learned_mixed": "learned+mixed: the mixed method with a shared base (SHARED_BASE_METHOD): every frame "
                                                   "starts from the density of a base kept from an earlier batch (the first warm-up "
                                                   "step, frames no timed step evaluates) and converges by FP32 perturbative density "
                                                   "steps around it (Riccati solve for |K| < 3e-2; no purification, no FP64 "
                                                   "eigensolve unless a frame falls back); the start density of every frame is the "
                                                   "learned linear response of the density to the QC coordinates and QC/MM "
                                                   "potentials (LinearResponseGuess, fitted to 2048 converged frames of another "
                                                   "seed), kept only where held-out validation shows SCF cycles saved"}[args.method],
                       "frame_sets": "a fresh seeded set of %d perturbed frames (sigma 0.02 A) per warm-up and timed step, the same "
                                     "sets for every method" % nF,
                       "perturbative_steps_per_frame": float(T["QC Densities Perturbative Steps"].mean()),
                       "density_tolerance": conv.densityTolerance, "mean_scf_cycles": ncyc_f,
                       "purification_steps_per_frame": pur_steps, "fp64_density_steps_per_frame": fp64_steps,
                       "scf_cta": scf_cta_layout(eng, T),
                       "l2": "working set > L2 (no flush needed)"},
            "e2e": {"value": e2e, "unit": UNIT, "ms_each": head["e2e_ms_each"], "h2d_bytes_per_step": int(head["frames_h"].numel() * 8),
                    "d2h_bytes_per_step": int(head["G"].nbytes + nF * (_native.NENERGY + 2 + nq) * 8),
                    "inputs": "each step's frames in their own pinned host buffer, allocated and copied once before timing",
                    "warmup_calls": args.warmup + 2},
            # per step: k_qcmm_potentials; k_pair_integrals, _ss, _sps, k_assemble_h; k_scf; k_pair_gradients, _ss, _sps,
            # k_reduce_gradients; k_qcmm_grad_qc, k_qcmm_grad_mm (or their FP32-pair forms)
            "gpu_launches": 12 * args.steps,
            "roofline": roofline(head, args.method != "fp64"),
            "kernel_rooflines": kernel_rooflines(head),
            "single_frame": single,
            "clocks": clk}
    if args.method != "fp64":
        # tensor-core part: SP2 iterations x k partial products x 2 N^3 algorithmic flops, over the purification
        # steps' device time (their clock64 cycles at the sampled SM clock)
        sp2 = float(T["QC Densities SP2 Iterations"].mean())
        pur_cycles = float(T["QC Densities Purification"].mean())
        mhz = (clk or {}).get("sm_mhz") or 2070.0
        t_pur = pur_cycles / (mhz * 1e6)
        tc_tf = (sp2 * 6 * 2.0 * N ** 3) / t_pur / 1e12 if t_pur > 0 else 0.0
        bf16 = bf16_peak / 152.0 / 2   # per SM, two SCF CTAs per SM share it
        line["roofline"]["tensor"] = {"achieved_per_cta": tc_tf, "unit": "TFLOP/s", "peak_per_cta": bf16,
                                      "frac": tc_tf / bf16 if bf16 else None,
                                      "note": "split-BF16 SP2 products of one frame's CTA (measured BF16 peak / 152 SMs / 2 CTAs per SM)"}
        dE = float(np.abs(head["E"] - plain["E"]).max()) / KJ
        dG = float(np.abs(head["G"] - plain["G"]).max()) / (KJ * 1.0e-10 / 5.291772083e-11)
        line["plain_fp64"] = {"value": n_total / (plain["ms"] * 1e-3), "ms_per_step": plain["ms"], "e2e": n_total / plain["e2e_s"],
                              "mean_scf_cycles": float(plain["ncyc"].mean()), "roofline": roofline(plain, False),
                              "kernel_rooflines": kernel_rooflines(plain)}
        if args.method == "learned_mixed":
            line["mixed"] = {"value": n_total / (mixed["ms"] * 1e-3), "ms_per_step": mixed["ms"], "e2e": n_total / mixed["e2e_s"],
                             "mean_scf_cycles": float(mixed["ncyc"].mean()),
                             "method": "MIXED_METHOD per frame (purification, one FP64 step, perturbative steps; no shared base)",
                             "phase_ms": mixed["phase_ms"]}
            line["learned_guess"] = guess_info
        line["accuracy_vs_plain_fp64"] = {"max_abs_dE_hartree": dE, "max_abs_dF_hartree_per_bohr": dG,
                                          "gate": "|dE| < 1e-6 Eh, |dF| < 1e-5 Eh/Bohr", "pass": bool(dE < 1e-6 and dG < 1e-5),
                                          "oracle": "each method's timed configuration is checked against the oracle frame by frame "
                                                    "in tests/test_gpu_timed_config.py"}
    if rank == 0 and not args.no_large:
        # config 4, the large QC/MM system over the whole GPU: a short Langevin trajectory per method
        line["large_qcmm"] = bench_large(args, md_steps=args.large_steps, md_warmup=3, cpu=not args.no_cpu_baseline)
    if rank == 0 and not args.no_cpu_baseline:
        n = min(nF, 96)
        cpu = CPUBaseline(Z, Q, sel, charge, 1)
        cpu.warm(frames)
        t, k, _ = cpu.run(frames[:n])
        line["cpu_baseline"] = {"value": k / t, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "%d frames, serial, cold E+grad each, oracle/mndo_oracle.c (C restatement; pDynamo's own "
                                          "core is not buildable on the GPU host)" % n}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
