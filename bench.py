"""E+F(+stress) throughput of the flare++ prediction path on GB300.

Workload (one step): the 32,768-atom two-species BCC alloy (32x32x16 cells,
a = 3.0 A, 0.08 A rattle, B2 chebyshev N=12 lmax=4, rc 5.5 A) against a sparse
GP with 2000 environments per species and power-2 NormalizedDotProduct
kernel, evaluated through its mapped coefficients (the pair style's form):
GPU neighbor list, B2 forward pass, split-fp16 tcgen05 contraction, adjoint
forces / virial.  Each step uses new positions (small seeded displacements).

Contract: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
prints one JSON line.  N > 1 runs as torchrun ranks, one independent replica
per GPU (the path is not sharded across GPUs); value = atoms/s of all ranks.
"""
import argparse
import json
import os
import re
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

UNIT = "atoms/s"
# name -> (metric, description, data, model builder, descriptor settings)
WORKLOADS = {
    "bcc_alloy_32k": (
        "E+F atoms/s at 32k atoms",
        "bcc_alloy_32k (32768 atoms, 2 species, B2 N=12 lmax=4, rc 5.5, "
        "2000 sparse/species, power 2)",
        "synthetic (seeded BCC alloy; model fitted to Lennard-Jones site energies)",
        "bcc_alloy_32k_recipe",
        dict(kind="B2", n_species=2, N=12, lmax=4, r1=0.0, rcut=5.5,
             cutoffs=np.full((2, 2), 5.5), cutoff_function="quadratic")),
    "bcc_alloy_16k": (
        "E+F atoms/s at 16k atoms",
        "bcc_alloy_16k (16384 atoms, the 32k workload's model on 32x16x16 cells; "
        "the small case for counter captures)",
        "synthetic (seeded BCC alloy; model fitted to Lennard-Jones site energies)",
        "bcc_alloy_16k_recipe",
        dict(kind="B2", n_species=2, N=12, lmax=4, r1=0.0, rcut=5.5,
             cutoffs=np.full((2, 2), 5.5), cutoff_function="quadratic")),
    "b3_fcc_1m": (
        "E+F atoms/s at 1M atoms (B3)",
        "b3_fcc_1m (1048576 atoms FCC Al 64^3 cells, B3 N=6 lmax=3, rc 5.0, "
        "500 sparse, power 2)",
        "synthetic (seeded FCC Al; model fitted to Lennard-Jones site energies)",
        "fcc_al_b3_1m_recipe",
        dict(kind="B3", n_species=1, N=6, lmax=3, r1=0.0, rcut=5.0,
             cutoffs=np.full((1, 1), 5.0), cutoff_function="quadratic")),
}
METRIC, WORKLOAD, DATA = WORKLOADS["bcc_alloy_32k"][:3]
SETTINGS = WORKLOADS["bcc_alloy_32k"][4]


def select_workload(name):
    global METRIC, WORKLOAD, DATA, SETTINGS
    METRIC, WORKLOAD, DATA, _, SETTINGS = WORKLOADS[name]


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def replica_time(ms_total, world, device=None):
    """Timed-region length of an N-replica run: the maximum over ranks (every
    rank processes its own copy of the workload; no data-path collective)."""
    if world <= 1:
        return ms_total
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms_total], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(n_atoms, steps, ms_total, world):
    """Whole-job atoms/s: all replicas' atoms over the slowest rank's time."""
    return world * n_atoms * steps / (ms_total / 1e3)


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML (the NVIDIA driver's
    libnvidia-ml, by ctypes) about every millisecond on a host thread, so that
    even a timed region of a few tens of milliseconds holds many samples.
    Reads only; the device is matched to the CUDA device by UUID."""
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown",
               0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, dev):
        import ctypes
        import torch
        self.ct = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        props = torch.cuda.get_device_properties(dev)
        found = False
        uuid = str(getattr(props, "uuid", ""))
        if uuid:
            uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
            found = self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.h)) == 0
        if not found and hasattr(props, "pci_bus_id"):
            bus = "%08x:%02x:%02x.0" % (getattr(props, "pci_domain_id", 0), props.pci_bus_id,
                                        props.pci_device_id)
            found = self.lib.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(),
                                                              ctypes.byref(self.h)) == 0
        if not found:
            n = ctypes.c_uint()
            if self.lib.nvmlDeviceGetCount_v2(ctypes.byref(n)) == 0 and n.value == 1:
                found = self.lib.nvmlDeviceGetHandleByIndex_v2(0, ctypes.byref(self.h)) == 0
        if not found:
            raise OSError("no NVML device matches CUDA device %s" % dev)
        try:
            self.reason_fn = self.lib.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self.reason_fn = self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        self.lib.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx))   # NVML_CLOCK_SM
        self.max_mhz = float(mx.value)
        self.samples = []
        self.stop_flag = False

    def read(self):
        clk, rs = self.ct.c_uint(), self.ct.c_ulonglong()
        if self.lib.nvmlDeviceGetClockInfo(self.h, 1, self.ct.byref(clk)) != 0:
            return None
        self.reason_fn(self.h, self.ct.byref(rs))
        return float(clk.value), int(rs.value)

    def _run(self):
        while not self.stop_flag:
            r = self.read()
            if r is not None:
                self.samples.append((time.perf_counter(),) + r)
            time.sleep(0.001)

    def start(self):
        self.t = threading.Thread(target=self._run, daemon=True)
        self.t.start()

    def stop(self, b, e):
        self.stop_flag = True
        self.t.join(timeout=2.0)
        inside = [x for x in self.samples if b <= x[0] <= e]
        window = "timed steps (NVML, ~1 ms period)"
        if not inside and self.samples:
            inside = [min(self.samples, key=lambda x: min(abs(x[0] - b), abs(x[0] - e)))]
            window = "adjacent to the timed steps (NVML)"
        reasons = sorted({nm for _, _, rs in inside for bit, nm in self.REASONS.items()
                          if rs & bit})
        self.lib.nvmlShutdown()
        return {"sm_mhz": float(np.median([c for _, c, _ in inside])) if inside else None,
                "sm_max_mhz": self.max_mhz, "reasons": reasons, "samples": len(inside),
                "window": window, "source": "nvml"}


class ClockSampler:
    """Clocks and throttle reasons sampled during the timed region: NVML every
    ~1 ms where the NVIDIA driver's NVML library loads, else nvidia-smi every
    100 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index, dev=None):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.nvml = None
        self.nvml_error = None
        if dev is not None:
            try:
                self.nvml = NvmlClocks(dev)
            except Exception as ex:  # no driver library or no match: nvidia-smi
                self.nvml = None
                self.nvml_error = str(ex)[:120]

    def start(self):
        if self.nvml is not None:
            self.nvml.start()
            return
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def wait_first(self, limit_s):
        t0 = time.perf_counter()
        while (self.nvml is None and self.proc is not None and not self.lines
               and time.perf_counter() - t0 < limit_s):
            time.sleep(0.02)

    def mark_begin(self):
        self.t_begin = time.perf_counter()

    def mark_end(self):
        self.t_end = time.perf_counter()

    def stop(self):
        if self.nvml is not None:
            return self.nvml.stop(getattr(self, "t_begin", -1e30), getattr(self, "t_end", 1e30))
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        # samples taken while the timed steps ran (one sample period of slack
        # on each side: nvidia-smi prints a sample up to 100 ms after taking it)
        b = getattr(self, "t_begin", -1e30)
        e = getattr(self, "t_end", 1e30) + 0.1
        inside = [(t, ln) for t, ln in self.lines if b <= t <= e]
        window = "timed steps"
        if not inside and self.lines:
            # timed steps shorter than the sample period: the samples just
            # before and just after them
            before = [x for x in self.lines if x[0] < b][-1:]
            after = [x for x in self.lines if x[0] > e][:1]
            inside = before + after
            window = "adjacent to the timed steps (shorter than a sample period)"
        for t, ln in inside:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "window": window,
                "source": "nvidia-smi" + (" (NVML: %s)" % self.nvml_error
                                          if self.nvml_error else "")}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0,
                "bf16_tflops_sustained": 1700.0}, "fallback"


PROFILE_FILES = {"bcc_alloy_32k": "contraction_bcc32k.txt",
                 "bcc_alloy_16k": None,
                 "b3_fcc_1m": "contraction_b3_fcc1m.txt"}


def profiled_traffic(workload="bcc_alloy_32k"):
    """DRAM bytes per contraction launch from the committed ncu summary."""
    if PROFILE_FILES.get(workload) is None:
        return None
    fn = os.path.join(ROOT, "profiles", PROFILE_FILES[workload])
    try:
        txt = open(fn).read()
    except OSError:
        return None
    m = re.search(r"dram_bytes_per_launch\s*=\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def build_workload(device, name="bcc_alloy_32k"):
    from flare_pp_gb300 import synth, Structure
    w = synth.model_from_recipe(getattr(synth, WORKLOADS[name][3])(), device=device)
    st = Structure(w["cell"], w["species"], w["positions"], SETTINGS["rcut"])
    return w, st


def config_of(noa, world):
    """The workload description both arms report (identical dicts)."""
    return {"workload": WORKLOAD, "n_atoms": int(noa), "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (per-step working set ~0.6 GB)"}


def step_positions(pos0, n, rank=0):
    """Per-step positions: the workload's frame with small seeded
    displacements (0.01 A), one frame per step."""
    rng = np.random.default_rng(1234 + rank)
    return [pos0 + rng.normal(scale=0.01, size=pos0.shape) for _ in range(n)]


def run_ours(args):
    import torch
    import torch.distributed as dist
    rank, world, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    from flare_pp_gb300 import _lib
    from flare_pp_gb300._lib import check, lib, ptr
    w, st = build_workload(dev, args.workload)
    gp = w["gp"]
    noa = st.noa
    gp._ensure_mapped()
    K, W = args.steps, args.warmup
    pos0 = np.asarray(w["positions"])
    disp = step_positions(pos0, K + W, rank)
    dpos = torch.tensor(np.stack(disp), dtype=torch.float64, device=dev)
    out_e = torch.zeros(1, dtype=torch.float64, device=dev)
    out_f = torch.zeros((noa, 3), dtype=torch.float64, device=dev)
    out_s = torch.zeros(6, dtype=torch.float64, device=dev)
    L = lib()
    mh, sh = gp._model.handle, st.handle
    stream = torch.cuda.current_stream(dev).cuda_stream

    def step(k, prec):
        check(L.fpp_structure_set_positions(sh, dpos[k].data_ptr(), 1, stream))
        check(L.fpp_predict_mapped(mh, sh, prec, out_e.data_ptr(), out_f.data_ptr(),
                                   out_s.data_ptr(), None, 1, stream))

    n_pairs = st.n_neighbors
    # ---- device-resident timing (value) ----
    clocks = ClockSampler(local, dev)
    clocks.start()
    for k in range(W):
        step(k, _lib.FPP_PREC_MIXED)
    clocks.wait_first(3.0)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks.mark_begin()
    torch.cuda.profiler.start()   # a profiler started with capture off sees only these steps
    ev0.record()
    for k in range(W, W + K):
        step(k, _lib.FPP_PREC_MIXED)
    ev1.record()
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    clocks.mark_end()
    clk = clocks.stop()
    free_b, total_b = torch.cuda.mem_get_info(dev)
    device_memory = {"used_gb": round((total_b - free_b) / 1e9, 2),
                     "total_gb": round(total_b / 1e9, 1),
                     "what": "device memory in use right after the timed steps: library "
                             "workspaces, model, inputs and torch buffers (other processes "
                             "on this GPU included)"}
    ms_total = replica_time(ev0.elapsed_time(ev1), world, dev)
    ms_step = ms_total / K
    value = replica_value(noa, K, ms_total, world)
    # ---- per-stage device times (separate pass: the event reads synchronize) ----
    check(L.fpp_structure_set_profiling(sh, 1))
    stage = np.zeros(4)
    n_stage = min(K, 20)
    for k in range(n_stage):
        step(W + k, _lib.FPP_PREC_MIXED)
        ms4 = np.zeros(4)
        check(L.fpp_structure_stage_times(sh, ptr(ms4)))
        stage += ms4
    check(L.fpp_structure_set_profiling(sh, 0))
    stage /= n_stage
    # ---- end-to-end through the public API with host buffers ----
    pinned = torch.from_numpy(np.stack(disp[:K])).pin_memory()
    he = np.zeros(1)
    hf_t = torch.zeros((noa, 3), dtype=torch.float64).pin_memory()  # pinned host forces
    hf = hf_t.numpy()
    hs = np.zeros(6)
    for k in range(min(2, K)):   # warm
        check(L.fpp_structure_set_positions(sh, pinned[k].data_ptr(), 0, stream))
        check(L.fpp_predict_mapped(mh, sh, _lib.FPP_PREC_MIXED, ptr(he), ptr(hf), ptr(hs),
                                   None, 0, stream))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(K):
        check(L.fpp_structure_set_positions(sh, pinned[k].data_ptr(), 0, stream))
        check(L.fpp_predict_mapped(mh, sh, _lib.FPP_PREC_MIXED, ptr(he), ptr(hf), ptr(hs),
                                   None, 0, stream))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * noa * K / e2e_s
    # ---- plain FP64 GPU form (same path, FP64 everywhere, cuBLAS DGEMM) ----
    step(0, _lib.FPP_PREC_FP64)
    torch.cuda.synchronize()
    k64 = max(1, min(5, K))
    f0 = torch.cuda.Event(enable_timing=True)
    f1 = torch.cuda.Event(enable_timing=True)
    f0.record()
    for k in range(k64):
        step(k, _lib.FPP_PREC_FP64)
    f1.record()
    torch.cuda.synchronize()
    fp64_ms = f0.elapsed_time(f1) / k64
    out_ae = torch.zeros(noa, dtype=torch.float64, device=dev)

    def outputs(prec):
        check(L.fpp_structure_set_positions(sh, dpos[0].data_ptr(), 1, stream))
        check(L.fpp_predict_mapped(mh, sh, prec, out_e.data_ptr(), out_f.data_ptr(),
                                   out_s.data_ptr(), out_ae.data_ptr(), 1, stream))
        torch.cuda.synchronize()
        return (out_e.item(), out_f.cpu().numpy().copy(), out_s.cpu().numpy().copy(),
                out_ae.cpu().numpy().copy())

    res64 = outputs(_lib.FPP_PREC_FP64)
    resmx = outputs(_lib.FPP_PREC_MIXED)
    err_fp64 = {"energy_per_atom_eV": abs(resmx[0] - res64[0]) / noa,
                "force_max_eV_per_A": float(np.abs(resmx[1] - res64[1]).max()),
                "stress_max_eV_per_A3": float(np.abs(resmx[2] - res64[2]).max())}
    # ---- roofline of the dominant kernel (the contraction) ----
    peaks, peak_src = measured_peaks()
    nd = gp._model.n_descriptors
    flop = 2.0 * noa * nd * nd            # algorithmic, counted once
    contract_ms = stage[2]
    achieved = flop / (contract_ms * 1e-3) / 1e12
    peak = float(peaks["bf16_tflops"])
    roof = {"kernel": "k_split_gemm_grouped (contraction P.beta, one persistent launch "
                      "over all species per step)",
            "bound": "tensor", "achieved": round(achieved, 2), "peak": peak,
            "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
            "peak_source": f"{peak_src} bf16 dense burst",
            "note": "algorithmic 2*n_atoms*n_d^2 FLOP per step; the split-fp16 form "
                    "issues 3 MMAs per product",
            "traffic": profiled_traffic(args.workload)}
    # ---- kernel form (predict_mean: E, F, S through the kernel against the
    # sparse set, FP64-accurate; its z and G products on the tensor cores) ----
    kernel_form, res_kf = None, None
    if rank == 0 and SETTINGS["kind"] == "B2":
        check(L.fpp_structure_set_positions(sh, dpos[0].data_ptr(), 1, stream))
        mean = np.zeros(1 + 3 * noa + 6)
        check(L.fpp_predict(mh, sh, mean.ctypes.data, None, stream))   # warm
        times = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            check(L.fpp_predict(mh, sh, mean.ctypes.data, None, stream))
            times.append(time.perf_counter() - t0)
        kf_ms = 1e3 * float(np.median(times))
        sp_arr = np.asarray(w["species"])
        n_sparse = [int(np.sum(np.asarray(w["fit"]["sparse"].n_clusters_by_type[s])))
                    for s in range(SETTINGS["n_species"])]
        kf_flop = float(sum(4.0 * n_sparse[s] * nd * np.sum(sp_arr == s)
                            for s in range(SETTINGS["n_species"])))
        kf_tf = kf_flop / (kf_ms * 1e-3) / 1e12
        kernel_form = {"ms": round(kf_ms, 2), "atoms_per_s": round(noa / (kf_ms * 1e-3), 1),
                       "what": "predict_mean E/F/S by the kernel form (FP64-accurate: z = "
                               "P Dhat^T and G = C Dhat on the tensor cores by exact fp16 "
                               "digit planes, FP64 descriptors and adjoint), host outputs",
                       "flop_per_atom": 4 * max(n_sparse) * nd,
                       "achieved_tflops_fp64_equivalent": round(kf_tf, 2),
                       "vs_fp64_dgemm_rate": round(kf_tf / 1.10, 2)}
        res_kf = (float(mean[0]), mean[1:1 + 3 * noa].reshape(-1, 3).copy(),
                  mean[1 + 3 * noa:].copy(), None)
    # ---- batched prediction: 256 uneven structures in one pass ----
    batched = None
    if rank == 0 and world == 1 and SETTINGS["kind"] == "B2" and not args.no_kuf:
        from flare_pp_gb300 import Structure
        from flare_pp_gb300 import synth as _synth
        cells = _synth.fcc_batch(n_structures=256, seed=404, lo=32, hi=512)
        strucs = [Structure(c, sp, p, SETTINGS["rcut"]) for c, sp, p in cells]
        n_b = sum(s.noa for s in strucs)
        gp.predict_mapped_batched(strucs, "mixed")    # warm (workspaces)
        times = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            gp.predict_mapped_batched(strucs, "mixed")
            times.append(time.perf_counter() - t0)
        tb = float(np.median(times))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for s in strucs:
            gp.predict_mapped(s, "mixed")
        t1 = time.perf_counter() - t0
        batched = {"what": "mapped E/F/S (mixed) of 256 FCC two-species cells of 32-512 "
                           "atoms in one pass (fpp_predict_mapped_batched), host outputs",
                   "structures": len(strucs), "atoms": int(n_b), "ms": round(1e3 * tb, 2),
                   "atoms_per_s": round(n_b / tb, 1), "one_by_one_ms": round(1e3 * t1, 2)}
    cpu, err_oracle = None, None
    if rank == 0 and not args.no_cpu:
        forms = {"mixed": resmx, "fp64_gpu": res64}
        if res_kf is not None:
            forms["kernel_form_fp64"] = res_kf
        cpu, err_oracle = oracle_check(w, disp[0], forms)
    # ---- energy variance and per-atom variances at this size (FP64) ----
    variance = None
    if SETTINGS["kind"] == "B2" and gp.R_inv is not None and gp.L_inv is not None:
        check(L.fpp_structure_set_positions(sh, dpos[0].data_ptr(), 1, stream))
        gp.predict_energy_uncertainty(st)          # warm (workspaces, L_inv upload)
        times = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            ev, vv, lv = gp.predict_energy_uncertainty(st)
            times.append(time.perf_counter() - t0)
        variance = {"ms": round(1e3 * float(np.median(times)), 2),
                    "what": "SOR energy variance and per-atom (L_inv) variances of all "
                            "atoms, FP64-accurate (kernel and L_inv products on the "
                            "tensor cores by exact fp16 digit planes), host outputs",
                    "energy_variance": vv, "local_variance_max": float(lv.max())}
        if rank == 0 and not args.no_cpu:
            variance["errors_vs_oracle"] = variance_check(w, disp[0], ev, vv, lv)
    kuf = None
    if rank == 0 and world == 1 and not args.no_kuf:
        try:
            kuf = kuf_batch_leg(args.kuf_structures)
        except Exception as e:      # recorded, never fatal to the headline line
            kuf = {"error": f"{type(e).__name__}: {e}"}
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": UNIT, "n_gpus": world,
        "steps": K, "warmup": W, "ms_per_step": round(ms_step, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp16x3/fp32 (descriptors fp32, contraction split-fp16, accumulate fp32)",
        "data": DATA,
        "config": config_of(noa, world),
        "workload_stats": {"n_pairs": int(n_pairs), "n_descriptors": nd},
        "stage_ms": {"neighbors": round(stage[0], 4), "descriptors": round(stage[1], 4),
                     "contraction": round(stage[2], 4), "adjoint": round(stage[3], 4)},
        "roofline": roof,
        "e2e": {"value": round(e2e_value, 1), "unit": UNIT,
                "h2d_bytes_per_step": int(noa * 3 * 8),
                "d2h_bytes_per_step": int(noa * 3 * 8 + 8 + 6 * 8)},
        "fp64_gpu": {"value": round(world * noa / (fp64_ms / 1e3), 1), "unit": UNIT,
                     "ms_per_step": round(fp64_ms, 3)},
        "errors_vs_oracle": err_oracle,
        "errors_vs_fp64_gpu": err_fp64,
        "variance": variance,
        "kernel_form": kernel_form,
        "batched_prediction": batched,
        "kuf_batched": kuf,
        "gpu_launches": int(K * launches_per_step(SETTINGS["n_species"])),
        "clocks": clk,
        "device_memory": device_memory,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def kuf_batch_leg(n_structures=256):
    """Training-side Kuf of the batched workload: 256 strained, rattled
    two-species FCC cells of 32-512 atoms (seed 404), N = 8, lmax = 3,
    rc 5.0, 1000 sparse environments drawn at random (seed 404), E, F and S
    label columns of every structure (labels are zeros: Kuf does not depend
    on them).  One fpp_kuf_batched call = the structures' FP64 descriptors
    (queued without host synchronization) and one persistent adjoint-route
    launch over all (structure, atom) items, tile shape from the library's
    autotuner (cached in a file).  Reported: the Kuf kernel's CUDA-event
    time on the second call, the whole call (host Kuf out), the tile shape,
    and the kernel's FP64 rate from its algorithmic FLOP count against the
    measured FP64 DGEMM rate of this GPU (1.10 TFLOP/s)."""
    import flare_pp_gb300 as fg
    from flare_pp_gb300 import synth
    rc = 5.0
    cells = synth.fcc_batch(n_structures=n_structures, seed=404, lo=32, hi=512)
    gb = fg.B2("chebyshev", "quadratic", [0, rc], [], [2, 8, 3])
    gb.store_dervs = False
    gp = fg.SparseGP([fg.NormalizedDotProduct(2.0, 2)], 0.001, 0.05, 0.006)
    strucs = []
    for cell, sp, pos in cells:
        s = fg.Structure(cell, sp, pos, rc, [gb])
        s.energy, s.forces, s.stresses = np.zeros(1), np.zeros(3 * len(sp)), np.zeros(6)
        gp.add_training_structure(s)
        strucs.append(s)
    rng = np.random.default_rng(404)
    allc = [(k, a) for k, (_, sp, _) in enumerate(cells) for a in range(len(sp))]
    pick = rng.choice(len(allc), min(1000, len(allc)), replace=False)
    for k in range(len(cells)):
        atoms = sorted(allc[p][1] for p in pick if allc[p][0] == k)
        if atoms:
            gp.add_specific_environments(strucs[k], atoms)
    sd, kern = gp.sparse_descriptors[0], gp.kernels[0]
    t0 = time.perf_counter()
    gp._kuf_batched(sd, kern)                   # first call: autotune or cached tiles
    first_s = time.perf_counter() - t0
    import torch
    torch.cuda.profiler.start()   # a profiler started with capture off sees this call
    t0 = time.perf_counter()
    Kuf = gp._kuf_batched(sd, kern)
    call_s = time.perf_counter() - t0
    torch.cuda.profiler.stop()
    ks, th, ms, items = gp.kuf_launch(len(gp._kuf_models) - 1)
    # algorithmic FP64 FLOP of the kernel per (atom i, sparse environment k of
    # i's species): z = dhat.phat (2 n_d), w (2 n_d), u = (W + W^T) c
    # (2 n_rad^2 H), and per pair f = u . dc/dr (4 N H + 8 H)
    N, lmax, ns = 8, 3, 2
    H = (lmax + 1) ** 2
    nr = ns * N
    nd = nr * (nr + 1) // 2 * (lmax + 1)
    n_sp = np.array(sd.n_clusters_by_type)
    flop = 0.0
    for s in strucs:
        cnt = s.neighbor_count.astype(np.float64)
        m = n_sp[np.asarray(s.species)].astype(np.float64)
        flop += float(np.sum(m * (4 * nd + 2 * nr * nr * H + cnt * (4 * N * H + 8 * H))))
    n_labels = Kuf.shape[1]
    achieved = flop / (ms / 1e3) / 1e12
    return {"workload": f"fcc_batch_{n_structures} ({n_structures} FCC two-species cells "
                        f"of 32-512 atoms, N=8 lmax=3 rc 5.0, {len(pick)} sparse)",
            "n_atoms": int(sum(len(sp) for _, sp, _ in cells)), "n_labels": int(n_labels),
            "work_items": int(items), "tiles": {"ks": ks, "threads": th},
            "tile_source": "autotuner (cached per device and descriptor shape)",
            "kernel_ms": round(ms, 2), "call_s": round(call_s, 3),
            "first_call_s": round(first_s, 3),
            "roofline": {"bound": "fp64", "achieved": round(achieved, 3),
                         "peak": 1.10, "unit": "TFLOP/s", "frac": round(achieved / 1.10, 3),
                         "peak_source": "measured cuBLAS DGEMM rate of this GPU",
                         "algorithmic_flop": flop}}


def launches_per_step(n_species):
    # neighbors: wrap_bin, bin_scatter, enum, nb_readback, compact_geom (which
    # also links reverse pairs) and two CUB exclusive scans of two kernels each
    # (compiled into the library); descriptors: forward; contraction: one
    # grouped split GEMM; adjoint: wu, pair_force, gather, reduce; outputs: finish
    return 9 + 1 + 1 + 4 + 1


def oracle_check(w, positions, results):
    """The FP64 C oracle (oracle/c/flare_oracle.c, whose pair-style math is
    pinned to the reference's lammps_descriptor.cpp) on the frame the GPU
    evaluated: the model's mapped coefficients computed on the host from its
    sparse set and weights, E/F/S of every atom (a sample of atoms, compared
    through their site energies, for frames above 65,536 atoms).  Returns
    (cpu_baseline, errors of each GPU form against it)."""
    from oracle import cfast
    from oracle import predict as opred
    from oracle.kernel import NormalizedDotProduct as ONDP
    fit = w["fit"]
    nd = fit["sparse"].n_descriptors
    B = opred.unpack_beta(ONDP(fit["sigma"], fit["power"]).compute_map_coeff_pow2(
        fit["sparse"], fit["alpha"]), nd)
    threads = cfast.max_threads()
    noa = len(w["species"])
    full = noa <= 65536
    atoms = None if full else np.arange(0, noa, noa // 4096)[:4096]
    t0 = time.perf_counter()
    ref = cfast.beta_form(w["cell"], w["species"], positions, SETTINGS, B, atoms=atoms,
                          n_threads=threads)
    dt = time.perf_counter() - t0
    n_eval = noa if full else len(atoms)
    cpu = {"value": round(n_eval / dt, 2), "unit": UNIT, "cores": threads, "kind": "port",
           "sample": (f"all {noa} atoms of one frame (E, F, S), {dt:.1f} s" if full else
                      f"{n_eval} of {noa} atoms (every {noa // 4096}th), {dt:.1f} s")}
    errs = {}
    for name, (e, f, s_, ae) in results.items():
        if full:
            errs[name] = {"energy_per_atom_eV": abs(e - ref["energy"]) / noa,
                          "force_max_eV_per_A": float(np.abs(f - ref["forces"]).max()),
                          "stress_max_eV_per_A3": float(np.abs(s_ - ref["stress"]).max())}
            if ae is not None:
                errs[name]["atom_energy_max_eV"] = float(np.abs(ae - ref["atom_energies"]).max())
        elif ae is None:
            continue
        else:
            errs[name] = {"atom_energy_max_eV": float(np.abs(ae[atoms] - ref["atom_energies"][atoms]).max()),
                          "sample_atoms": n_eval}
    errs["oracle"] = "oracle/c/flare_oracle.c, FP64, same frame and model"
    return cpu, errs


def variance_check(w, positions, energy, energy_variance, local, n_sample=512):
    """The same model's energy (k_E . alpha), SOR energy variance
    (|R_inv^T k_E|^2) and per-atom variances (k(i,i) - |L_inv k_i|^2) in FP64
    on the host: descriptors from the C oracle, kernel columns and products in
    numpy; per-atom variances on a seeded sample of atoms."""
    from oracle import cfast
    fit = w["fit"]
    sd = fit["sparse"]
    sig2, pw = fit["sigma"] ** 2, fit["power"]
    sp = np.asarray(w["species"])
    p, nrm = cfast.b2_descriptors(w["cell"], sp, positions, SETTINGS,
                                  n_threads=cfast.max_threads())
    n = sd.n_clusters
    kE = np.zeros(n)
    rng = np.random.default_rng(99)
    sample = np.sort(rng.choice(len(sp), min(n_sample, len(sp)), replace=False))
    ksamp = np.zeros((n, len(sample)))
    for s_ in range(sd.n_types):
        D = np.asarray(sd.descriptors[s_])
        dn = np.asarray(sd.descriptor_norms[s_])
        okd = dn >= 1e-8
        Dh = np.zeros_like(D)
        Dh[okd] = D[okd] / dn[okd, None]
        idx = np.nonzero((sp == s_) & (nrm >= 1e-8))[0]
        off = sd.cumulative_type_count[s_]
        Ph = p[idx] / nrm[idx, None]
        Z = Dh @ Ph.T
        kE[off:off + len(dn)] = sig2 * (Z ** pw).sum(axis=1) * okd
        for c, i in enumerate(sample):
            if sp[i] == s_ and nrm[i] >= 1e-8:
                ksamp[off:off + len(dn), c] = sig2 * (Dh @ (p[i] / nrm[i])) ** pw * okd
    e_ref = kE @ fit["alpha"]
    v_ref = float(np.sum((np.asarray(fit["R_inv"]).T @ kE) ** 2))
    Q = np.asarray(fit["L_inv"]) @ ksamp
    loc_ref = np.where(nrm[sample] >= 1e-8, sig2, 0.0) - np.einsum("ij,ij->j", Q, Q)
    return {"energy_eV": abs(energy - e_ref),
            "energy_variance_rel": abs(energy_variance - v_ref) / max(abs(v_ref), 1e-300),
            "local_variance_max_abs": float(np.abs(local[sample] - loc_ref).max()),
            "sample_atoms": int(len(sample)),
            "oracle": "FP64 host (C oracle descriptors, numpy products), same model"}


def run_reference(args):
    """The reference's CPU algorithm for the path on the host cores: the
    oracle's C restatement of pair_flare.cpp's per-atom form (the
    reference's own sources need Eigen 3.3.7 and nlohmann_json and are not
    present on the GPU machines), all host threads.  Everything here is host
    code: the workload frames come from the numpy recipe, the model is
    fitted in FP64 by the oracle (oracle/site_fit.py) and the GPU library is
    never loaded.  Each step evaluates E, F, S of all atoms of a new frame
    when K such steps fit in about two and a half minutes, else the first n
    atoms of it (stated in cpu_baseline.sample)."""
    rank, world, local = dist_env()
    if rank != 0:
        return
    from flare_pp_gb300 import synth      # numpy-only recipes; loads no library
    from oracle import cfast, site_fit
    r = getattr(synth, WORKLOADS[args.workload][3])()
    settings = SETTINGS
    threads = cfast.max_threads()
    t_fit = time.perf_counter()
    ys = [synth.lennard_jones(c, p)[3] for (c, _, p) in r["frames"]]
    B, _, _ = site_fit.fit_site_energy_beta(r["frames"], settings, ys, r["n_sparse"],
                                            sigma=r["sigma"], power=r["power"], seed=r["seed"],
                                            n_threads=threads)
    t_fit = time.perf_counter() - t_fit
    noa = len(r["species"])
    K, W = args.steps, args.warmup
    disp = step_positions(np.asarray(r["positions"]), K + W)
    probe = np.arange(min(noa, 512))
    t0 = time.perf_counter()
    cfast.beta_form(r["cell"], r["species"], disp[0], settings, B, atoms=probe,
                    n_threads=threads)
    per_atom = (time.perf_counter() - t0) / len(probe)
    budget = 150.0
    n_step = noa if per_atom * noa * K <= budget else max(512, int(budget / (K * per_atom)))
    atoms = None if n_step >= noa else np.arange(n_step)
    for k in range(W):   # untimed warm-up steps on a small sample
        cfast.beta_form(r["cell"], r["species"], disp[k], settings, B, atoms=probe,
                        n_threads=threads)
    t0 = time.perf_counter()
    for k in range(W, W + K):
        cfast.beta_form(r["cell"], r["species"], disp[k], settings, B, atoms=atoms,
                        n_threads=threads)
    dt = time.perf_counter() - t0
    n_eval = noa if atoms is None else n_step
    value = n_eval * K / dt
    sample = (f"all {noa} atoms per step (E, F, S of a new frame)" if atoms is None else
              f"the first {n_step} of {noa} atoms per step")
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 2), "unit": UNIT,
            "n_gpus": world, "steps": K, "warmup": W,
            "ms_per_step": round(dt / K * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": DATA, "config": config_of(noa, world),
            "cpu_baseline": {"value": round(value, 2), "unit": UNIT, "cores": threads,
                             "kind": "port", "sample": sample + f"; model fitted on the host "
                             f"in {t_fit:.0f} s"},
            "e2e": {"value": round(value, 2), "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def measure_matmul_peaks(n=8192, seconds=4.0):
    """FP64 and TF32 matmul peaks of this GPU, the way the bf16 peak is
    measured: torch.matmul of n^3 (2 n^3 FLOP), best of 10 (burst) and back to
    back for `seconds` (sustained), CUDA events.  The FP64 figures bound the
    FP64 path (cuBLAS DGEMM contraction, training solve, uncertainties)."""
    import torch
    dev = torch.device("cuda", 0)
    out = {}
    for name, dtype, tf32 in (("fp64", torch.float64, False), ("tf32", torch.float32, True)):
        torch.backends.cuda.matmul.allow_tf32 = tf32
        a = torch.randn(n, n, dtype=dtype, device=dev)
        b = torch.randn(n, n, dtype=dtype, device=dev)
        c = torch.empty(n, n, dtype=dtype, device=dev)
        for _ in range(3):
            torch.matmul(a, b, out=c)
        torch.cuda.synchronize()
        best = float("inf")
        for _ in range(10):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        reps = max(1, int(seconds / best))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            torch.matmul(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        sus = e0.elapsed_time(e1) * 1e-3 / reps
        flop = 2.0 * n ** 3
        out[name] = {"tflops_burst": flop / best / 1e12, "tflops_sustained": flop / sus / 1e12,
                     "n": n, "sustained_reps": reps}
        del a, b, c
    torch.backends.cuda.matmul.allow_tf32 = False
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-kuf", action="store_true",
                    help="skip the batched-Kuf (training) leg")
    ap.add_argument("--kuf-structures", type=int, default=256,
                    help="structures of the batched-Kuf leg (256: the full workload)")
    ap.add_argument("--workload", default="bcc_alloy_32k", choices=sorted(WORKLOADS))
    ap.add_argument("--measure-peaks", action="store_true",
                    help="print the FP64 and TF32 matmul peaks and exit")
    args = ap.parse_args()
    if args.measure_peaks:
        print(json.dumps(measure_matmul_peaks()))
        return
    select_workload(args.workload)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
