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
on the host cores (one frame per process, all cores) on a bounded sample of the same frames.
"""

import argparse, json, os, subprocess, sys, threading, time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

import numpy as np

# DRAM bytes (read + write) of one k_scf launch on this workload (304 frames), from the ncu captures summarised
# in profiles/k_scf_dram_304frames.md; per launch, like `achieved` (mixed: this build; plain: an earlier build).
K_SCF_DRAM_BYTES_304 = {"mixed": 8.59e9 + 5.12e9, "fp64": 4.85e9 + 4.10e9}

METRIC = "QC/MM E+grad evals/s at |dE|<1e-6 Eh (AM1 RHF, 65 QC atoms in 4000 TIP3P waters, ABFS 8/12 A)"
UNIT = "evals/s"
KJ = 2625.5


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
    Z, X, Q, sel, charge = workloads.qcmm_water_box(seed=seed)
    frames = workloads.perturbed_frames(X, n_frames, sigma=0.02, seed=11)
    return Z, X, Q, sel, charge, frames


def cpu_reference_sample(Z, Q, sel, charge, frames, n_sample, processes):
    """Oracle E+grad on n_sample frames, `processes` at a time (spawned workers). Returns (seconds, n)."""
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    args = [(list(Z), Q, sel, charge, frames[f]) for f in range(n_sample)]
    t0 = time.perf_counter()
    if processes == 1:
        for a in args:
            _oracle_eval(a)
    else:
        with ctx.Pool(processes) as pool:
            pool.map(_oracle_eval, args)
    return time.perf_counter() - t0, n_sample


def _oracle_eval(args):
    sys.path.insert(0, HERE)
    from oracle import oracle as O
    Z, Q, sel, charge, X = args
    nq = len(sel)
    knots = O.abfs_knots(8.0, 12.0)
    phi, _, _ = O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], knots=knots)
    r = O.System(O.Hamiltonian("am1", Z[:nq]), Z[:nq], charge=charge).energy(X[:nq], phi=phi)
    O.qcmm("abfs", X[:nq], X[nq:], Q[nq:], qcq=r["charges"], knots=knots)
    return r["eelectronic"]


def run_reference(args):
    Z, X, Q, sel, charge, frames = workload(max(args.frames, args.reference_sample))
    cores = os.cpu_count() or 1
    n = min(len(frames), max(cores, args.reference_sample))
    times = []
    for s in range(args.warmup + args.steps):
        t, k = cpu_reference_sample(Z, Q, sel, charge, frames, n, cores)
        if s >= args.warmup:
            times.append(t)
    value = n / (sum(times) / len(times))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded water box, perturbed frames)",
            "config": {"workload": "qcmm_water_box_am1_abfs", "qc_atoms": len(sel), "mm_atoms": len(Z) - len(sel),
                       "frames_per_step": n},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": "%d frames per step, one frame per process, oracle/mndo_oracle.c" % n},
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
    convs = {"fp64": DIISSCFConverger(),
             "mixed": DIISSCFConverger(densityStep="purification", purificationProducts=6, purificationSwitch=1e-5)}
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
    MIXED = dict(densityStep="purification", purificationProducts=6, purificationSwitch=1e-5)

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
    snap = dict(xyz=ho.xyz.clone(), vel=ho.vel.clone(), acc=ho.acc.clone(), hist=[h.clone() for h in ho.history], n=ho.n_step)
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
        m.xyz.copy_(snap["xyz"]); m.vel.copy_(snap["vel"]); m.acc.copy_(snap["acc"]); m.n_step = snap["n"]
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
    ap.add_argument("--workload", default="qcmm_water_box", choices=["qcmm_water_box", "water_clusters", "qcmm_md"],
                    help="the QC/MM water box (the headline metric), 512 independent PM3 water clusters in one launch, or "
                         "Langevin dynamics of water-box replicas with the learned start density trained on trajectories")
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
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            run_reference(args)
        return

    import torch
    from pdynamo_mirror_gb300 import NBModelABFS, QCModelMNDO, System, _native
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    dev = torch.device("cuda")
    Z, X, Q, sel, charge, frames = workload(args.frames, seed=1 + rank)
    from pdynamo_mirror_gb300 import DIISSCFConverger
    METHODS = {"fp64": dict(densityStep="fp64"),
               "mixed": dict(densityStep="purification", purificationProducts=6, purificationSwitch=1e-5)}
    METHODS["learned_mixed"] = METHODS["mixed"]
    guess_info = {}

    def train_guess(s, eng):
        """The learned start density, trained on frames the SCF converges here (a seed apart from the timed
        frames); returns the model and what it achieved on held-out frames."""
        from pdynamo_mirror_gb300 import LearnedDensityGuess
        t0 = time.perf_counter()
        from pdynamo_mirror_gb300 import workloads
        tr = workloads.perturbed_frames(X, 2048, sigma=0.02, seed=101 + rank)
        qc_t, mm_t, q_t, _ = s._device_inputs(tr)
        phis, dens = [], []
        for s0 in range(0, len(tr), 256):
            r = eng.run(qc_t[s0:s0 + 256].contiguous(), s.qcModel.converger, mm_t[s0:s0 + 256].contiguous(), q_t, s.nbModel,
                        gradients=False, warm_start=False)
            phis.append(r["phi"].clone()); dens.append(eng.density.clone())
        phi, P = torch.cat(phis), torch.cat(dens)
        g = LearnedDensityGuess(eng, seed=0)
        hist = g.fit(qc_t, phi, P, epochs=40, batch=32, lr=1e-3, seed=0)
        hist += g.fit(qc_t, phi, P, epochs=20, batch=32, lr=2e-4, seed=1)
        torch.cuda.synchronize()
        return g, {"training_frames": len(tr), "epochs": 60, "train_seconds": time.perf_counter() - t0,
                   "loss_first_last": [hist[0], hist[-1]]}

    def measure(method, timed_clocks):
        s = System(Z, X, mmCharges=Q)
        s.electronicState.charge = charge
        s.DefineQCModel(QCModelMNDO("am1", converger=DIISSCFConverger(**METHODS[method])), qcSelection=sel)
        s.DefineNBModel(NBModelABFS(innerCutoff=8.0, outerCutoff=12.0))
        eng = s.engine()
        qc, mm, q, mm_idx = s._device_inputs(frames)
        conv, nb = s.qcModel.converger, s.nbModel
        guess = None
        if method == "learned_mixed":
            guess, info = train_guess(s, eng)
            s.DefineDensityGuess(guess)
            # held-out validation (frames of their own seed): the guess stays on only if it saves SCF cycles
            from pdynamo_mirror_gb300 import workloads
            qc_v, mm_v, q_v, _ = s._device_inputs(workloads.perturbed_frames(X, 256, sigma=0.02, seed=201 + rank))
            info.update(guess.validate(qc_v, conv, mm_v, q_v, nb))
            info["used_in_timed_steps"] = guess.enabled
            guess_info.update(info)

        def step():
            return eng.run(qc, conv, mm, q, nb, gradients=True, warm_start=False, guess=guess)

        for _ in range(args.warmup):
            r = step()
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
        e0.record(stream)
        for _ in range(args.steps):
            r = step()
        e1.record(stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ms = e0.elapsed_time(e1) / args.steps
        clk = clocks.stop() if clocks else None
        timers = eng.timings(len(frames))
        # the dominant kernel alone: k_scf through pdg_scf on the integrals the last step left in the
        # workspace (same frames, cold guess), CUDA events on the launching stream
        k0, k1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        scf_times = []
        for _ in range(3):
            k0.record(stream)
            eng.scf(conv, phi=r["phi"], use_density=False)
            k1.record(stream)
            torch.cuda.synchronize()
            scf_times.append(k0.elapsed_time(k1))
        if world > 1:
            t = torch.tensor([ms], device=dev)
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            ms = float(t.item())
        # e2e through the public API: frames from pinned host memory in, energies and gradients out
        frames_h = torch.from_numpy(np.ascontiguousarray(frames)).pin_memory()
        te = []
        for k in range(2 + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            E, G, terms = s.EnergyBatch(frames_h, doGradients=True, warmStart=False)
            torch.cuda.synchronize()
            if k >= 2:
                te.append(time.perf_counter() - t0)
        return dict(ms=ms, clk=clk, scf_ms=float(np.median(scf_times)), e2e_s=sum(te) / len(te), E=E, G=G,
                    ncyc=r["ncycles"].cpu().numpy(), timers=timers, eng=eng, conv=conv, frames_h=frames_h)

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
    bf16_peak = peaks().get("bf16_tflops", 1925.7)

    def roofline(h, mixed):
        """FP64 roofline of the method's k_scf (its FP64 algorithmic flops over the event-timed launch, against
        cuBLAS DGEMM measured here) and, for the mixed method, the composite: the time its FP64, FP32 and tensor work
        would take at the three measured peaks over the measured time."""
        f64, f32, tc = scf_work(h["timers"], N, kv, len(frames), mixed)
        t = h["scf_ms"] * 1e-3
        r = {"bound": "fp64", "kernel": "k_scf", "achieved": f64 / t / 1e12, "peak": fp64_peak, "unit": "TFLOP/s",
             "frac": f64 / t / 1e12 / fp64_peak,
             "traffic": K_SCF_DRAM_BYTES_304["mixed" if mixed else "fp64"] if len(frames) == 304 else None,
             "note": "FP64 algorithmic flops of the density steps over the k_scf launch (%.2f ms, %d frames); peak = cuBLAS DGEMM "
                     "4096^3 measured in this run (of measured; MEASURED_PEAKS.json has no FP64 figure)" % (h["scf_ms"], len(frames))}
        if mixed:
            t_ideal = f64 / (fp64_peak * 1e12) + f32 / (fp32_peak * 1e12) + tc / (bf16_peak * 1e12)
            r["composite"] = {"t_ideal_ms": t_ideal * 1e3, "t_measured_ms": h["scf_ms"], "frac": t_ideal / t,
                              "fp64_tflop": f64 / 1e12, "fp32_tflop": f32 / 1e12, "tensor_tflop": tc / 1e12,
                              "fp32_peak_tflops": fp32_peak, "bf16_peak_tflops": bf16_peak,
                              "note": "the mixed SCF spreads its work over the FP64 pipe (FP64 base steps), the FP32 pipe (perturbative "
                                      "steps, commutators) and the tensor cores (SP2): time at the three measured peaks (FP32: cuBLAS "
                                      "SGEMM 4096^3 without TF32, measured here; BF16: MEASURED_PEAKS.json) over the measured launch"}
        return r
    clk = head["clk"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": head["ms"], "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded water box, perturbed frames)",
            "config": {"workload": "qcmm_water_box_am1_abfs", "qc_atoms": len(sel), "mm_atoms": len(Z) - len(sel),
                       "basis_functions": N, "frames_per_step": len(frames),
                       "method": {"fp64": "plain FP64",
                                  "mixed": "mixed: split-BF16 SP2 purification on tcgen05 (6 partial products, FP32 accumulation) until the RMS density change < 1e-5, then FP64",
                                  "learned_mixed": "learned+mixed: per-pair MLP start density (kept only where held-out validation shows "
                                                   "SCF cycles saved, else the diagonal guess), then the mixed SCF"}[args.method],
                       "density_tolerance": conv.densityTolerance, "mean_scf_cycles": ncyc_f,
                       "purification_steps_per_frame": pur_steps, "fp64_density_steps_per_frame": fp64_steps,
                       "scf_cta": scf_cta_layout(eng, T),
                       "l2": "working set > L2 (no flush needed)"},
            "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": int(head["frames_h"].numel() * 8),
                    "d2h_bytes_per_step": int(head["G"].nbytes + len(frames) * (_native.NENERGY + 2 + len(sel)) * 8)},
            "gpu_launches": 8 * args.steps,
            "roofline": roofline(head, args.method != "fp64"),
            "clocks": clk}
    if args.method != "fp64":
        # tensor-core part: SP2 iterations x k partial products x 2 N^3 algorithmic flops, over the purification
        # steps' device time (their clock64 cycles at the sampled SM clock)
        sp2 = float(T["QC Densities SP2 Iterations"].mean())
        pur_cycles = float(T["QC Densities Purification"].mean())
        mhz = (clk or {}).get("sm_mhz") or 2070.0
        t_pur = pur_cycles / (mhz * 1e6)
        tc_tf = (sp2 * 6 * 2.0 * N ** 3) / t_pur / 1e12 if t_pur > 0 else 0.0
        pk = peaks()
        bf16 = pk.get("bf16_tflops", 1900.0) / 152.0 / 2   # per SM, two SCF CTAs per SM share it
        line["roofline"]["tensor"] = {"achieved_per_cta": tc_tf, "unit": "TFLOP/s", "peak_per_cta": bf16,
                                      "frac": tc_tf / bf16 if bf16 else None,
                                      "note": "split-BF16 SP2 products of one frame's CTA (measured BF16 peak / 152 SMs / 2 CTAs per SM)"}
        dE = float(np.abs(head["E"] - plain["E"]).max()) / KJ
        dG = float(np.abs(head["G"] - plain["G"]).max()) / (KJ * 1.0e-10 / 5.291772083e-11)
        line["plain_fp64"] = {"value": n_total / (plain["ms"] * 1e-3), "ms_per_step": plain["ms"], "e2e": n_total / plain["e2e_s"],
                              "mean_scf_cycles": float(plain["ncyc"].mean()), "roofline": roofline(plain, False)}
        if args.method == "learned_mixed":
            line["mixed"] = {"value": n_total / (mixed["ms"] * 1e-3), "ms_per_step": mixed["ms"], "e2e": n_total / mixed["e2e_s"],
                             "mean_scf_cycles": float(mixed["ncyc"].mean())}
            line["learned_guess"] = guess_info
        line["accuracy_vs_plain_fp64"] = {"max_abs_dE_hartree": dE, "max_abs_dF_hartree_per_bohr": dG,
                                          "gate": "|dE| < 1e-6 Eh, |dF| < 1e-5 Eh/Bohr", "pass": bool(dE < 1e-6 and dG < 1e-5)}
    if rank == 0 and not args.no_cpu_baseline:
        n = min(len(frames), 96)
        t, k = cpu_reference_sample(list(Z), Q, sel, charge, frames, n, 1)
        line["cpu_baseline"] = {"value": k / t, "unit": UNIT, "cores": 1, "kind": "port",
                                "sample": "%d frames, serial, oracle/mndo_oracle.c (C restatement; pDynamo's own core is not buildable on the GPU host)" % n}
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
