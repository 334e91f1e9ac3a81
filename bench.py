"""Benchmark of the SICC GB300 receive path (one JSON line on stdout).

Workload (default, ``bp_osd_128_64``): the QC (128,64) code, BPSK over AWGN,
65,536 frames per batch at Eb/N0 = 2 dB and 3 dB, layered normalized min-sum
(alpha 0.75, at most 20 iterations, early stop) with order-2 OSD (1 + 64 +
2016 tests) on every frame whose syndrome fails.  One step decodes one batch
at each Eb/N0 (131,072 codewords, 8.39 Mbit of information), each Eb/N0 point
on its own decoder and CUDA stream (two receive chains: one chain's BP runs
beside the other's OSD).  Inputs are
seeded synthetic LLRs; several distinct batches are kept resident on the GPU
(larger than L2 together) and cycled between steps.

Metric: information-bit throughput in Mbit/s (sum of k over decoded codewords
divided by the timed wall time), with the frame error rate of each Eb/N0
point reported beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's CPU decoder for the same workload
on the host cores: its flooding normalized min-sum (restated bit-exactly in
the oracle) plus the oracle's OSD restatement, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import json
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "sicc-baseband-proto_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

EBN0 = (2.0, 3.0)
BATCH = 65536
RESIDENT_BATCHES = 4  # per Eb/N0: 8 x 33.5 MB of LLRs resident, > 129 MB of L2 together
ITERS, ALPHA = 20, 0.75
OSD_ORDER, OSD_FLIP, OSD_TESTS = 2, 64, 4096
WORKLOAD = "bp_osd_128_64"
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")
TRAFFIC = os.path.join(ROOT, "profiles", "bp_layered_128_64_traffic.json")
KERNEL_TRAFFIC = os.path.join(ROOT, "profiles", "kernel_traffic.json")


def traffic_for(kernel, units):
    """DRAM bytes of `kernel` for `units` (frames or codewords) from its ncu capture, or None."""
    try:
        with open(KERNEL_TRAFFIC) as f:
            return int(round(json.load(f)[kernel]["bytes_per_unit"] * units))
    except Exception:
        return None


KERNEL_ISSUE = os.path.join(ROOT, "profiles", "kernel_issue.json")


def issue_roofline(kernel, units, launch_ms, launches, sm_mhz):
    """Issue-bound roofline of `kernel`: warp instructions per unit (one ncu capture, see
    KERNEL_ISSUE) x units processed / kernel time, against SMs x 4 schedulers x 1 warp
    instruction per cycle at the sampled SM clock.  None when the kernel has no capture."""
    try:
        with open(KERNEL_ISSUE) as f:
            rec = json.load(f)[kernel]
    except Exception:
        return None
    import torch
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    mhz = sm_mhz or 2070.0
    peak = sms * 4 * mhz * 1e6 / 1e9  # G warp instructions / s
    achieved = rec["warp_inst_per_unit"] * units / (launch_ms * launches * 1e-3) / 1e9
    return {"bound": "issue", "kernel": kernel, "unit": "G warp instructions/s", "achieved": round(achieved, 2),
            "peak": round(peak, 2), "frac": round(achieved / peak, 4),
            "warp_inst_per_unit": rec["warp_inst_per_unit"], "per": rec["unit"], "units": int(units),
            "avg_launch_ms": round(launch_ms, 4), "peak_source": f"{sms} SMs x 4 schedulers at {mhz:.0f} MHz",
            "capture": rec.get("capture")}


def peaks():
    try:
        with open(PEAKS) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------- CPU baseline
_CPU_CODE = {}


def _cpu_worker(args):
    llr, iters, alpha = args
    if "oc" not in _CPU_CODE:  # code tables built once per worker process
        from oracle import Oracle
        from sicc_gb300 import codes
        c = codes.short_code()
        oc = Oracle().code(c.n, c.m, c.row_ptr, c.col_ind)
        _CPU_CODE.update(oc=oc, table=oc.systematic_parity())
    oc, table = _CPU_CODE["oc"], _CPU_CODE["table"]
    t0 = time.perf_counter()
    info, used = oc.bp_osd_batch(llr, schedule=0, max_iter=iters, alpha=alpha, osd_order=OSD_ORDER,
                                 osd_max_flip=OSD_FLIP, osd_max_tests=OSD_TESTS, table=table)
    return time.perf_counter() - t0, info, used


def _cpu_mixed_worker(args):
    """One code's sample of the mixed workload through the restated layered BP + OSD (host core)."""
    n, m, row_ptr, col_ind, llr, iters, order = args
    from oracle import Oracle
    oc = Oracle().code(n, m, row_ptr, col_ind)
    table = oc.systematic_parity()
    t0 = time.perf_counter()
    oc.bp_osd_batch(llr, schedule=3, max_iter=iters, alpha=ALPHA, osd_order=order, osd_max_flip=OSD_FLIP,
                    osd_max_tests=OSD_TESTS, table=table)
    return time.perf_counter() - t0


def _cpu_ofdm_worker(args):
    """Frames of the OFDM workload through the restated CPU receive chain: sync, demod, layered decode."""
    iq, noise_var, iters = args
    from oracle import Oracle
    from sicc_gb300 import codes, ofdm
    o = Oracle()
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    ph = o.phy(t)
    oc = o.code(code.n, code.m, code.row_ptr, code.col_ind)
    blocks = t.coded_bits // code.n
    t0 = time.perf_counter()
    for x in iq:
        r = o.sync_earliest(ph, x)
        if r[0] != 1:
            continue
        llr = o.demod_frame(ph, x[r[1]: r[1] + t.frame_len], r[4], noise_var)
        for b in range(blocks):
            oc.layered(llr[b * code.n: (b + 1) * code.n], iters, ALPHA)
    return time.perf_counter() - t0


def fer_parity_point(sent, ref_info, gpu_info, gpu_flood_info):
    """Error rates of the reference decoder and the GPU decoders on identical frames."""
    from sicc_gb300 import errstats
    ref = errstats.rate_summary(ref_info, sent)
    lay = errstats.rate_summary(gpu_info, sent)
    pair = errstats.mcnemar(errstats.frame_errors(gpu_info, sent) > 0, errstats.frame_errors(ref_info, sent) > 0)
    lo, hi = ref["fer_ci95"]
    return {"frames": ref["frames"],
            "reference": {"fer": ref["fer"], "fer_ci95": [round(lo, 6), round(hi, 6)], "ber": ref["ber"],
                          "ber_ci95": [round(x, 7) for x in ref["ber_ci95"]]},
            "gpu_layered": {"fer": lay["fer"], "ber": lay["ber"],
                            "fer_vs_reference_ci": "inside" if lo <= lay["fer"] <= hi else
                            ("below" if lay["fer"] < lo else "above"),
                            "ber_vs_reference_ci": "inside" if errstats.inside(lay["ber"], ref["ber_ci95"]) else
                            ("below" if lay["ber"] < ref["ber_ci95"][0] else "above"),
                            "frames_only_gpu_fails": pair["only_a"], "frames_only_reference_fails": pair["only_b"],
                            "mcnemar_p": round(pair["p_value"], 6)},
            "gpu_flooding_bit_exact": bool(np.array_equal(gpu_flood_info, ref_info))}


def cpu_decode(pool, workers, llr):
    chunks = np.array_split(llr, 4 * workers)
    t0 = time.perf_counter()
    res = pool.map(_cpu_worker, [(c, ITERS, ALPHA) for c in chunks])
    wall = time.perf_counter() - t0
    info = np.concatenate([r[1] for r in res])
    used = np.concatenate([r[2] for r in res])
    return wall, info, used


def max_over_ranks(value, device):
    """The largest of every rank's `value` (all ranks get it): a step's time is the slowest rank's."""
    import torch
    import torch.distributed as dist
    dist.barrier()
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(units_per_rank, world, steps, elapsed_ms):
    """Whole-job throughput: the units every rank processed over the slowest rank's time."""
    return world * units_per_rank * steps / (elapsed_ms * 1e-3)


def make_inputs(batch, n_batches, seed0):
    from sicc_gb300 import channel, codes
    code = codes.short_code()
    out = {}
    for e in EBN0:
        out[e] = [channel.awgn_llrs(code, batch, e, seed=seed0 + int(e * 100) + 7 * b) for b in range(n_batches)]
    return code, out


# -------------------------------------------------------------- clock sampler
class ClockSampler:
    def __init__(self, index=0):
        self.index, self.rows, self.proc = index, [], None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm = [float(r[0]) for r in self.rows if len(r) >= 7 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 7 and r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 7 for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(sm)}


def _bp_kernel_name(code):
    """The layered BP kernel the library picks for a QC code (its launcher's rule)."""
    d = next(x for x in (6, 8, 10, 12, 14, 16, 27) if int(np.max(np.diff(code.row_ptr))) <= x)
    group = 1
    while group < code.z and group < 32:
        group *= 2
    rows_per_lane = -(-code.z // group)
    if d <= 8 and code.mb * rows_per_lane <= 4:
        return f"bp_layered_reg_kernel<{d},4>"
    return f"bp_layered_kernel<{d}>"


# ------------------------------------------------------------------- our arm
def run_ours(args, rank, world):
    import torch
    from sicc_gb300 import fec

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", dev))

    code, inputs = make_inputs(BATCH, RESIDENT_BATCHES, seed0=1000 * (rank + 1))
    # CPU baseline pool: spawned before the first GPU call of this process
    pool = workers = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        workers = os.cpu_count() or 1
        pool = mp.get_context("spawn").Pool(workers)

    stream = torch.cuda.current_stream()
    d_llr = {e: [torch.from_numpy(x[2]).cuda() for x in inputs[e]] for e in EBN0}
    # one decoder and stream per Eb/N0 point (two receive chains): one chain's BP overlaps the
    # other's OSD
    chain = {}
    for e in EBN0:
        chain[e] = dict(
            dec=fec.StreamBpOsdDecoder(code, max_batch=BATCH, max_iter=ITERS, normalization=ALPHA, offset=0.0,
                                       damping=0.0, min_abs_llr_accept=0.0, osd_order=OSD_ORDER,
                                       osd_max_flip=OSD_FLIP, osd_max_tests=OSD_TESTS),
            stream=torch.cuda.Stream(),
            out=[torch.zeros((BATCH, code.k), dtype=torch.uint8, device="cuda")] +
                [torch.zeros(BATCH, dtype=torch.uint8, device="cuda") for _ in range(3)])  # info, ok, used, iters

    # launch shapes picked by the autotuner on each chain's first batch (cached for the
    # reference-API decoders of the end-to-end leg, which decode the same code with the same settings)
    shapes = {}
    for e in EBN0:
        if args.no_tune:
            shapes[f"{e:g}dB"] = chain[e]["dec"].shape()
        else:
            res = chain[e]["dec"].autotune(d_llr[e][0], reps=3)
            shapes[f"{e:g}dB"] = dict(res.best, tuned_ms=round(res.best_ms, 4), default_ms=round(res.default_ms, 4),
                                      trials=len(res.trials))

    def step(s):
        for e in EBN0:
            c = chain[e]
            c["dec"].decode_device_batch(d_llr[e][s % RESIDENT_BATCHES], *c["out"], stream=c["stream"])

    def fork(ev):
        for e in EBN0:
            chain[e]["stream"].wait_event(ev)

    def join():
        for e in EBN0:
            ev = torch.cuda.Event()
            ev.record(chain[e]["stream"])
            stream.wait_event(ev)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    for e in EBN0:
        chain[e]["dec"].set_timing(True)
    clocks = ClockSampler(dev)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    fork(ev0)
    for s in range(args.steps):
        step(s)
    join()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    calls = bp_ms = osd_ms = osd_cw = 0
    for e in EBN0:
        k_calls, k_bp, k_osd, k_cw = chain[e]["dec"].kernel_ms()
        chain[e]["dec"].set_timing(False)
        calls, bp_ms, osd_ms, osd_cw = calls + k_calls, bp_ms + k_bp, osd_ms + k_osd, osd_cw + k_cw
    # edge updates of the timed launches: the batches cycle, so count each resident batch's
    # iterations (decoded again below for the error rates) by how often it ran
    timed_edges = 0
    if world > 1:
        elapsed_ms = max_over_ranks(elapsed_ms, "cuda")

    # frame error rate and iterations on one resident batch per Eb/N0
    fer, mean_iter, osd_frac = {}, {}, {}
    gpu_info = {}
    edge_updates = 0
    for e in EBN0:
        info_true = inputs[e][0][0]
        d_info, d_ok, d_used, d_it = chain[e]["out"]
        chain[e]["dec"].decode_device_batch(d_llr[e][0], d_info, d_ok, d_used, d_it, stream=stream)
        torch.cuda.synchronize()
        got = d_info.cpu().numpy()
        gpu_info[e] = got
        fer[f"{e:g}dB"] = float(np.mean(np.any(got != info_true, axis=1)))
        it = d_it.cpu().numpy().astype(np.int64)
        mean_iter[f"{e:g}dB"] = float(it.mean())
        osd_frac[f"{e:g}dB"] = float(d_used.cpu().numpy().mean())
        edge_updates += int(it.sum()) * code.edges
        for r in range(RESIDENT_BATCHES):  # every resident batch's iterations, weighted by its timed runs
            runs = sum(1 for s_ in range(args.steps) if s_ % RESIDENT_BATCHES == r)
            if runs:
                chain[e]["dec"].decode_device_batch(d_llr[e][r], d_info, d_ok, d_used, d_it, stream=stream)
                torch.cuda.synchronize()
                timed_edges += runs * int(d_it.cpu().numpy().astype(np.int64).sum()) * code.edges

    # the reference's schedule on the GPU: flooding min-sum + OSD on the best-syndrome posterior
    # (the reference decoder's arithmetic, bit for bit): its throughput and its bits on batch 0
    flood = {e: fec.StreamBpOsdDecoder(code, max_batch=BATCH, max_iter=ITERS, normalization=ALPHA, offset=0.0,
                                       damping=0.0, min_abs_llr_accept=0.0, schedule=0, osd_order=OSD_ORDER,
                                       osd_max_flip=OSD_FLIP, osd_max_tests=OSD_TESTS) for e in EBN0}

    def flood_step(s):
        for e in EBN0:
            flood[e].decode_device_batch(d_llr[e][s % RESIDENT_BATCHES], *chain[e]["out"], stream=chain[e]["stream"])

    for s in range(min(args.warmup, 3)):
        flood_step(s)
    torch.cuda.synchronize()
    ev0.record(stream)
    fork(ev0)
    for s in range(args.steps):
        flood_step(s)
    join()
    ev1.record(stream)
    torch.cuda.synchronize()
    flood_ms = ev0.elapsed_time(ev1)
    if world > 1:
        flood_ms = max_over_ranks(flood_ms, "cuda")
    flood_info = {}
    for e in EBN0:
        d_info = chain[e]["out"][0]
        flood[e].decode_device_batch(d_llr[e][0], d_info, stream=stream)
        torch.cuda.synchronize()
        flood_info[e] = d_info.cpu().numpy()

    bits_per_step = len(EBN0) * BATCH * code.k
    value = world * bits_per_step * args.steps / (elapsed_ms * 1e-3) / 1e6

    # ---- end to end through the reference-facing C ABI with host buffers ----
    e2e = None
    if not args.no_e2e:
        # one reference-API decoder per receive chain (Eb/N0 point), as the device-timed step
        dec_api = {e: fec.StreamBpOsdDecoder(code, max_batch=BATCH, min_batch=BATCH, max_iter=ITERS,
                                             normalization=ALPHA, offset=0.0, damping=0.0, min_abs_llr_accept=0.0,
                                             osd_order=OSD_ORDER, osd_max_flip=OSD_FLIP, osd_max_tests=OSD_TESTS)
                   for e in EBN0}
        pinned = {}
        for e in EBN0:
            pinned[e] = []
            for b in range(2):
                h = torch.empty((BATCH, code.n), dtype=torch.float32, pin_memory=True)
                h.numpy()[:] = inputs[e][b][2]
                pinned[e].append(h.numpy())
        # the reference's streaming use (L:3309-3432, the receive loop L:11482-11633): frames are
        # submitted as they arrive and results polled as they come back.  Each receive chain (Eb/N0
        # point) has its own host thread, as a receiver runs one decode thread per chain: step s
        # submits the chain's frames (a submit returns once its host copy is done), then collects
        # the chain's step s - 2, so the GPU always holds a queued batch while the host uploads and
        # copies results out; the last steps are flushed and drained before the clock stops.  Every step's LLRs cross
        # host->device and its information bits device->host inside the timed region.  The C ABI
        # calls release the interpreter lock, so the chains' host work runs side by side.
        bufs = {e: dec_api[e].poll_buffers(BATCH) for e in EBN0}
        blocks = np.arange(BATCH, dtype=np.uint32)

        def e2e_chain(e, i, steps, errors):
            try:
                def collect():
                    got = 0
                    while got < BATCH:
                        got += len(dec_api[e].poll(BATCH - got, bufs[e])[0])
                lag = 2  # batches in flight per chain beyond the one being collected (the ring holds 4)
                for s in range(steps):
                    dec_api[e].submit(pinned[e][s % 2], np.full(BATCH, 2 * s + i, np.uint64), blocks)
                    if s >= lag:
                        collect()
                dec_api[e].flush()
                for _ in range(min(lag, steps)):
                    collect()
            except Exception as exc:  # reported by the caller
                errors.append(exc)

        def e2e_run(steps):
            errors = []
            threads = [threading.Thread(target=e2e_chain, args=(e, i, steps, errors)) for i, e in enumerate(EBN0)]
            for t in threads:
                t.start()
            for t in threads:
                t.join()
            if errors:
                raise errors[0]

        e2e_run(min(args.warmup, 2))
        torch.cuda.synchronize()
        # a streaming receiver runs in steady state: at least 40 steps, so the pipeline's fill and
        # drain (two steps in flight per chain) are a small part of the timed region
        e2e_steps = max(args.steps, 40)
        t0 = time.perf_counter()
        e2e_run(e2e_steps)
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": round(world * bits_per_step * e2e_steps / e2e_s / 1e6, 3), "unit": "Mbit/s",
               "steps": e2e_steps,
               "h2d_bytes_per_step": len(EBN0) * BATCH * code.n * 4,
               "d2h_bytes_per_step": len(EBN0) * BATCH * (code.k + 1),
               "api": "cuda_osd_submit_codewords + cuda_osd_poll_ready, one stream decoder and one host thread "
                      "per Eb/N0 chain, streaming (step s is submitted while steps s-1 and s-2 decode and are "
                      "collected; flush + drain at the end), pinned host LLRs"}

    # ---- roofline of the dominant kernel (layered BP) ----
    peak, peak_kind = peaks()
    bytes_per_cw = 4 * code.n + code.k + 3  # LLR in; info bits, success, OSD flag, iterations out
    avg_bp_ms = bp_ms / max(calls, 1)
    alg_bytes = BATCH * bytes_per_cw
    achieved = alg_bytes / (avg_bp_ms * 1e-3) / 1e9
    traffic = None
    try:  # dram bytes per codeword from one ncu capture, scaled to this launch's frames
        with open(TRAFFIC) as f:
            traffic = round(json.load(f)["dram_bytes_per_codeword"] * BATCH)
    except Exception:
        pass
    roofline_bp = {"bound": "hbm", "achieved": round(achieved, 2), "peak": peak, "unit": "GB/s",
                   "frac": round(achieved / peak, 5), "traffic": traffic, "peak_source": peak_kind,
                   "kernel": _bp_kernel_name(code),
                   "algorithmic_bytes_per_launch": alg_bytes,
                   "avg_launch_ms": round(avg_bp_ms, 4),
                   "edge_updates_per_s": round(edge_updates / len(EBN0) / (avg_bp_ms * 1e-3), 1),
                   "note": "BP is issue-bound (messages and row tables in registers, posteriors in shared memory); "
                           "roofline_issue.bp has the issue-bound form"}
    # the OSD kernel's HBM view (the failed codewords' posteriors in, their bits out)
    avg_osd_ms = osd_ms / max(calls, 1)
    osd_per_launch = osd_cw / max(calls, 1)
    osd_bytes = int(osd_per_launch * (4 * code.n + code.k + 1))
    osd_achieved = osd_bytes / (avg_osd_ms * 1e-3) / 1e9 if avg_osd_ms > 0 else 0.0
    roofline_osd = {"bound": "hbm", "achieved": round(osd_achieved, 2), "peak": peak, "unit": "GB/s",
                    "frac": round(osd_achieved / peak, 5),
                    "traffic": traffic_for("osd_kernel<2,2>", osd_per_launch),
                    "peak_source": peak_kind, "kernel": "osd_kernel<2,2>",
                    "algorithmic_bytes_per_launch": osd_bytes, "avg_launch_ms": round(avg_osd_ms, 4),
                    "note": "OSD is issue-bound (integer ALU); roofline_issue.osd has the issue-bound form"}
    # `roofline` is the kernel with the larger share of the step's kernel time, the other beside it
    osd_share = osd_ms / max(osd_ms + bp_ms, 1e-9)
    roofline, roofline_other = (roofline_osd, roofline_bp) if osd_ms >= bp_ms else (roofline_bp, roofline_osd)
    roofline = dict(roofline, share_of_kernel_time=round(max(osd_share, 1.0 - osd_share), 3),
                    dominant="the larger share of the step's kernel time; both kernels are issue-bound, so their "
                             "HBM fractions are small by design: roofline_issue has the issue-bound forms")
    # issue-bound rooflines of the step's two kernels (OSD is the larger share of it)
    roofline_issue = {
        "osd": issue_roofline("osd_kernel<2,2>", osd_cw, osd_ms / max(calls, 1), calls, clk.get("sm_mhz")),
        "bp": issue_roofline(_bp_kernel_name(code), timed_edges, avg_bp_ms, calls, clk.get("sm_mhz"))}
    # the whole step: both kernels' instructions over the step time.  Each kernel's own figure above
    # divides by its launch time while the other chain's kernels share the SMs, so it understates
    if roofline_issue["osd"] and roofline_issue["bp"]:
        total = (roofline_issue["osd"]["warp_inst_per_unit"] * osd_cw
                 + roofline_issue["bp"]["warp_inst_per_unit"] * timed_edges)
        peak_i = roofline_issue["bp"]["peak"]
        achieved_i = total / (elapsed_ms * 1e-3) / 1e9  # this GPU's instructions over the (slowest) step
        roofline_issue["step"] = {"bound": "issue", "unit": "G warp instructions/s", "achieved": round(achieved_i, 2),
                                  "peak": peak_i, "frac": round(achieved_i / peak_i, 4),
                                  "warp_instructions_per_step": int(total / args.steps),
                                  "note": "BP + OSD instructions of the timed steps over the timed region"}

    # ---- CPU baseline: the reference decoder on the same frames, and the error-rate parity ----
    cpu = fer_parity = None
    if pool is not None:
        wall = 0.0
        fer_parity = {}
        for e in EBN0:
            info_true = inputs[e][0][0]
            w, ref_info, _ = cpu_decode(pool, workers, inputs[e][0][2])
            wall += w
            fer_parity[f"{e:g}dB"] = fer_parity_point(info_true, ref_info, gpu_info[e], flood_info[e])
        pool.close()
        fer_parity["reference_schedule_on_gpu"] = {
            "value": round(world * bits_per_step * args.steps / (flood_ms * 1e-3) / 1e6, 3), "unit": "Mbit/s",
            "what": "flooding min-sum + OSD on the best-syndrome posterior (bit-exact with the reference decoder), "
                    "same chains and batches as the headline step"}
        cpu = {"value": round(len(EBN0) * BATCH * code.k / wall / 1e6, 4), "unit": "Mbit/s",
               "cores": workers, "kind": "port",
               "sample": f"the first resident batch at each of 2 and 3 dB ({BATCH} frames each, the frames of "
                         f"fer_parity): the reference decoder (flooding min-sum alpha 0.75, 20 iterations, "
                         f"order-2 OSD on the best-syndrome posterior), {workers} worker processes"}

    if rank == 0:
        line = {"metric": "info-bit Mbps BP+OSD (128,64), Eb/N0 2 and 3 dB", "value": round(value, 3),
                "unit": "Mbit/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded BPSK/AWGN LLRs)",
                "config": {"workload": WORKLOAD, "code": "QC (128,64) 4x8 base Z=16", "frames_per_batch": BATCH,
                           "chains": "one decoder and CUDA stream per Eb/N0 point",
                           "ebn0_db": list(EBN0), "bp": f"layered NMS alpha {ALPHA}, <= {ITERS} iterations",
                           "osd": f"order {OSD_ORDER}, {1 + OSD_FLIP + OSD_FLIP * (OSD_FLIP - 1) // 2} tests",
                           "l2": f"{2 * RESIDENT_BATCHES} resident batches of 33.5 MB cycled (> L2)",
                           "parallelism": f"replicas x{world}", "launch_shapes": shapes},
                "fer": fer, "fer_parity": fer_parity, "mean_iterations": mean_iter, "osd_fraction": osd_frac,
                "gpu_launches": args.steps * len(EBN0) * 2, "clocks": clk, "roofline": roofline,
                "roofline_issue": roofline_issue, "roofline_other": roofline_other,
                "e2e": e2e, "cpu_baseline": cpu}
    if world > 1:
        dist.destroy_process_group()
    return line if rank == 0 else None


# ------------------------------------------------------- OFDM receive workload
OFDM_SNRS = (8.0, 12.0, 16.0)
OFDM_FRAMES = 256
OFDM_ITERS = 25


def run_ofdm(args, rank, world):
    """Sync + demod + decode of 256-frame batches of the 16-QAM OFDM workload."""
    import torch
    from sicc_gb300 import codes, fec, ofdm
    from sicc_gb300.pipeline import RxPipeline, SYNC_RECORD

    dev = int(os.environ.get("LOCAL_RANK", 0))
    # CPU baseline pool: spawned before the first GPU call of this process
    pool = workers = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        workers = os.cpu_count() or 1
        pool = mp.get_context("spawn").Pool(workers)
    torch.cuda.set_device(dev)
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    frames = args.ofdm_frames
    per_snr = 2  # resident batches per SNR point: 6 x 34 MB of IQ > L2
    batches = {}
    for i, snr in enumerate(OFDM_SNRS):
        gen = ofdm.FrameGenerator(t, code, seed=500 + 10 * i + rank)
        batches[snr] = [gen.batch(frames, snr_db=snr, cfo_subcarriers=0.1, max_offset=200, rayleigh_taps=6)
                        for _ in range(per_snr)]
    blocks = t.coded_bits // code.n
    pipes = {snr: RxPipeline(t, code.n, code.k, blocks, float(np.float32(np.mean(batches[snr][0].noise_var))),
                             max_batch_frames=frames) for snr in OFDM_SNRS}
    stream = torch.cuda.current_stream()
    d_iq = {snr: [torch.from_numpy(b.iq).cuda() for b in batches[snr]] for snr in OFDM_SNRS}
    L = batches[OFDM_SNRS[0]][0].iq.shape[1]
    # one receive chain (decoder, buffers, CUDA stream) per SNR point: one chain's sync and demod
    # run beside another's decode
    chain = {snr: dict(
        dec=fec.CsrBpDecoder.for_code(code, max_batch=frames * blocks, max_iter=OFDM_ITERS, normalization=ALPHA),
        stream=torch.cuda.Stream(),
        llr=torch.zeros((frames * blocks, code.n), dtype=torch.float32, device="cuda"),
        bits=torch.zeros((frames * blocks, code.n), dtype=torch.uint8, device="cuda"),
        ok=torch.zeros(frames * blocks, dtype=torch.uint8, device="cuda"),
        sync=torch.zeros(frames * SYNC_RECORD.itemsize, dtype=torch.uint8, device="cuda"),
        d_in=torch.empty((frames, L), dtype=torch.complex64, device="cuda"),
        h_out=torch.empty((frames * blocks, code.n), dtype=torch.uint8, pin_memory=True)) for snr in OFDM_SNRS}

    def run_chain(snr, iq, st):
        c = chain[snr]
        pipes[snr].demod_batch(iq, L, L, frames, c["llr"], c["sync"], st)
        c["dec"].decode_device_batch(c["llr"], c["bits"], c["ok"], None, None, stream=st)

    # BP launch shapes tuned on each chain's own demodulated LLRs (the first batch)
    shapes = {}
    for snr in OFDM_SNRS:
        c = chain[snr]
        pipes[snr].demod_batch(d_iq[snr][0], L, L, frames, c["llr"], c["sync"], stream)
        torch.cuda.synchronize()
        if args.no_tune:
            shapes[f"{snr:g}dB"] = c["dec"].shape()
        else:
            res = c["dec"].autotune(c["llr"], reps=2)
            shapes[f"{snr:g}dB"] = dict(res.best, tuned_ms=round(res.best_ms, 4), default_ms=round(res.default_ms, 4))

    def step(s):
        for snr in OFDM_SNRS:
            run_chain(snr, d_iq[snr][s % per_snr], chain[snr]["stream"])

    def fork(ev):
        for snr in OFDM_SNRS:
            chain[snr]["stream"].wait_event(ev)

    def join():
        for snr in OFDM_SNRS:
            ev = torch.cuda.Event()
            ev.record(chain[snr]["stream"])
            stream.wait_event(ev)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    fork(ev0)
    for s in range(args.steps):
        step(s)
    join()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    info_bits = len(OFDM_SNRS) * frames * blocks * code.k
    value = world * info_bits * args.steps / (elapsed_ms * 1e-3) / 1e6

    # kernel split of one step (chains one after another), FER per SNR point
    fer, cer, sync_ms, demod_ms, bp_ms = {}, {}, 0.0, 0.0, 0.0
    good_cw = 0  # correctly decoded codewords of the first batch at every SNR
    for snr in OFDM_SNRS:
        b = batches[snr][0]
        c = chain[snr]
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pipes[snr].demod_batch(d_iq[snr][0], L, L, frames, c["llr"], c["sync"], stream)
        e0.record(stream)
        c["dec"].decode_device_batch(c["llr"], c["bits"], c["ok"], None, None, stream=stream)
        e1.record(stream)
        torch.cuda.synchronize()
        a, d = pipes[snr].last_batch_ms()
        sync_ms += a
        demod_ms += d
        bp_ms += e0.elapsed_time(e1)
        info = c["bits"].cpu().numpy()[:, : code.k].reshape(frames, -1)
        fer[f"{snr:g}dB"] = float(np.mean(np.any(info != b.info, axis=1)))
        cw_ok = ~np.any(info.reshape(frames, blocks, code.k) != b.info.reshape(frames, blocks, code.k), axis=2)
        cer[f"{snr:g}dB"] = float(1.0 - cw_ok.mean())
        good_cw += int(cw_ok.sum())

    # end to end: pinned host IQ -> device, search + demod + decode, decoded bits -> host
    h_iq = {snr: torch.empty((frames, L), dtype=torch.complex64, pin_memory=True) for snr in OFDM_SNRS}
    for snr in OFDM_SNRS:
        h_iq[snr].numpy()[:] = batches[snr][0].iq
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.steps):
        for snr in OFDM_SNRS:
            c = chain[snr]
            with torch.cuda.stream(c["stream"]):
                c["d_in"].copy_(h_iq[snr], non_blocking=True)
                run_chain(snr, c["d_in"], c["stream"])
                c["h_out"].copy_(c["bits"], non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    cpu = None
    if pool is not None:  # 64 frames per SNR point through the restated CPU receiver, all host cores
        sample = min(64, frames)
        tasks = []
        for snr in OFDM_SNRS:
            b = batches[snr][1]  # 256 frames per batch by default
            nv = float(np.float32(np.mean(b.noise_var)))
            for part in np.array_split(np.arange(sample), max(1, workers // len(OFDM_SNRS))):
                if len(part):
                    tasks.append((b.iq[part], nv, OFDM_ITERS))
        c0 = time.perf_counter()
        pool.map(_cpu_ofdm_worker, tasks)
        cs = time.perf_counter() - c0
        pool.close()
        cpu = {"value": round(len(OFDM_SNRS) * sample * blocks * code.k / cs / 1e6, 4), "unit": "Mbit/s",
               "cores": workers, "kind": "port",
               "sample": f"{sample} frames at each SNR: the restated CPU receiver (sync, demod, 30 layered decodes "
                         "of 25 iterations per frame; oracle/sicc_oracle.c)"}

    peak, peak_kind = peaks()
    demod_bytes = frames * (8 * t.cfg.num_symbols * t.cfg.nfft + 4 * blocks * code.n)
    maxdeg = int(np.max(np.diff(code.row_ptr)))
    bp_name = f"bp_layered_kernel<{next(d for d in (6, 8, 10, 12, 14, 16, 27) if maxdeg <= d)}>"
    kern = {"sync_kernel": sync_ms, "demod_kernel": demod_ms, bp_name: bp_ms}
    top = max(kern, key=kern.get)
    achieved = demod_bytes / (demod_ms / len(OFDM_SNRS) * 1e-3) / 1e9
    line = {"metric": "info-bit Mbps OFDM RX (sync+demod+decode), 16-QAM, (1024,512)", "value": round(value, 3),
            "unit": "Mbit/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded 16-QAM OFDM frames, 6-tap Rayleigh)",
            "config": {"workload": "ofdm_rx_1024_512", "frames_per_batch": frames, "snr_db": list(OFDM_SNRS),
                       "chains": "one pipeline, decoder and CUDA stream per SNR point",
                       "fft": 1024, "cp": 72, "active_sc": 600, "symbols": 14, "code": "QC (1024,512) Z=64",
                       "bp_iterations": OFDM_ITERS, "codewords_per_frame": blocks,
                       "l2": "6 resident batches of 34 MB cycled (> L2)", "launch_shapes": shapes},
            "fer": fer, "codeword_error_rate": cer,
            "goodput": {"value": round(value * good_cw / (len(OFDM_SNRS) * frames * blocks), 3), "unit": "Mbit/s",
                        "what": "information bits of correctly decoded codewords per second (the value times the "
                                "correct fraction of the first batch at each SNR); frames the receiver does not "
                                "find count as lost, as in the reference receiver"},
            "kernel_ms_per_step": {k: round(v, 4) for k, v in kern.items()}, "dominant_kernel": top,
            "gpu_launches": args.steps * len(OFDM_SNRS) * 3, "clocks": clk,
            "roofline": {"bound": "hbm", "kernel": "demod_kernel", "achieved": round(achieved, 2), "peak": peak,
                         "unit": "GB/s", "frac": round(achieved / peak, 5), "traffic": traffic_for("demod_kernel", frames),
                         "peak_source": peak_kind,
                         "algorithmic_bytes_per_launch": demod_bytes},
            "e2e": {"value": round(world * info_bits * args.steps / e2e_s / 1e6, 3), "unit": "Mbit/s",
                    "h2d_bytes_per_step": len(OFDM_SNRS) * frames * L * 8,
                    "d2h_bytes_per_step": len(OFDM_SNRS) * frames * blocks * code.n},
            "cpu_baseline": cpu}
    return line if rank == 0 else None


# ------------------------------------------------------ OFDM transmit workload
def run_ofdm_tx(args, rank, world):
    """Encode + modulate 256-frame batches of the 16-QAM OFDM workload (the GPU transmitter)."""
    import torch
    from sicc_gb300 import codes, ofdm
    from sicc_gb300.pipeline import RxPipeline

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    frames = args.ofdm_frames
    per_step = len(OFDM_SNRS)  # batches per step, as the receive workload
    resident = 6                # 6 x 35.5 MB of output frames cycled (> L2)
    blocks = t.coded_bits // code.n
    G = np.ascontiguousarray(np.concatenate([np.eye(code.k, dtype=np.uint8), codes.gf2_parity_matrix(code)], 1))
    pipe = RxPipeline(t, code.n, code.k, blocks, 1e-3, max_batch_frames=frames)
    pipe.upload_tx_tables(generator_kn=G)
    rng = np.random.default_rng(900 + rank)
    info = [rng.integers(0, 2, size=(frames, blocks * code.k), dtype=np.uint8) for _ in range(resident)]
    d_info = [torch.from_numpy(x).cuda() for x in info]
    L = t.frame_len
    d_out = [torch.empty((frames, L), dtype=torch.complex64, device="cuda") for _ in range(resident)]
    stream = torch.cuda.current_stream()

    def step(s):
        for b in range(per_step):
            i = (s * per_step + b) % resident
            pipe.tx_batch(d_info[i], frames, d_out[i], stream=stream)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for s in range(args.steps):
        step(s)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    info_bits = per_step * frames * blocks * code.k
    value = world * info_bits * args.steps / (elapsed_ms * 1e-3) / 1e6

    # one batch alone: the roofline of the transmitter (encode + symbol kernels)
    reps = 10
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for r in range(reps):
        pipe.tx_batch(d_info[r % resident], frames, d_out[r % resident], stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    batch_ms = e0.elapsed_time(e1) / reps
    tx_bytes = frames * (blocks * code.k + 2 * blocks * code.n + 8 * L)  # info in, coded out + in, frame out

    # end to end: pinned host info bits -> device -> frames -> pinned host, the step's batches on
    # their own CUDA streams so one batch's copies overlap another's kernels
    lanes = [dict(stream=torch.cuda.Stream(),
                  h_info=torch.empty((frames, blocks * code.k), dtype=torch.uint8, pin_memory=True),
                  d_in=torch.empty((frames, blocks * code.k), dtype=torch.uint8, device="cuda"),
                  h_out=torch.empty((frames, L), dtype=torch.complex64, pin_memory=True)) for _ in range(per_step)]
    for ln in lanes:
        ln["h_info"].numpy()[:] = info[0]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.steps):
        for b, ln in enumerate(lanes):
            with torch.cuda.stream(ln["stream"]):
                ln["d_in"].copy_(ln["h_info"], non_blocking=True)
                pipe.tx_batch(ln["d_in"], frames, d_out[b], stream=ln["stream"])
                ln["h_out"].copy_(d_out[b], non_blocking=True)
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0

    cpu = None
    if not args.no_cpu_baseline and rank == 0:  # the restated transmitter on one host core
        import tx_oracle
        cfg = t.cfg
        sample = 4
        c0 = time.perf_counter()
        cw = tx_oracle.encode_generator(info[1][:sample].reshape(-1, code.k), G).reshape(sample, -1)
        tx_oracle.tx_frames(cw, nfft=cfg.nfft, cp=cfg.cp, num_symbols=cfg.num_symbols, active_sc=cfg.active_sc,
                            bps=cfg.bits_per_symbol, used_bins=t.used_bins, pilot_symbols=t.pilot_symbols,
                            data_symbols=t.data_symbols, pilot_grid=t.pilot_grid, preamble=t.preamble,
                            amplitude=cfg.amplitude)
        cs = time.perf_counter() - c0
        cpu = {"value": round(sample * blocks * code.k / cs / 1e6, 4), "unit": "Mbit/s", "cores": 1, "kind": "port",
               "sample": f"{sample} frames: generator encode + grid + inverse FFT + frame (oracle/tx_oracle.py, NumPy)"}

    peak, peak_kind = peaks()
    achieved = tx_bytes / (batch_ms * 1e-3) / 1e9
    line = {"metric": "info-bit Mbps OFDM TX (encode+modulate+IFFT+frame), 16-QAM, (1024,512)",
            "value": round(value, 3), "unit": "Mbit/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded information bits)",
            "config": {"workload": "ofdm_tx_1024_512", "frames_per_batch": frames, "batches_per_step": per_step,
                       "fft": 1024, "cp": 72, "active_sc": 600, "symbols": 14, "code": "QC (1024,512) Z=64",
                       "codewords_per_frame": blocks, "l2": "6 resident output batches of 35.5 MB cycled (> L2)"},
            "batch_ms": round(batch_ms, 4),
            "gpu_launches": args.steps * per_step * 2, "clocks": clk,
            "roofline": {"bound": "hbm", "kernel": "tx_encode + tx_symbol_kernel", "achieved": round(achieved, 2),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5),
                         "traffic": traffic_for("tx_encode + tx_symbol_kernel", frames),
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": tx_bytes},
            "e2e": {"value": round(world * info_bits * args.steps / e2e_s / 1e6, 3), "unit": "Mbit/s",
                    "h2d_bytes_per_step": per_step * frames * blocks * code.k,
                    "d2h_bytes_per_step": per_step * frames * L * 8},
            "cpu_baseline": cpu}
    return line if rank == 0 else None


# ------------------------------------------------------ real-time ingest workload
def run_ingest(args, rank, world):
    """A continuous C3-PHY stream through the device ring: push 16,384-sample blocks, step after each."""
    import torch
    from sicc_gb300 import codes, ofdm
    from sicc_gb300.ingest import Ingest
    from sicc_gb300.pipeline import RxPipeline

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    code = codes.ofdm_code()
    blocks = t.coded_bits // code.n
    fl = t.frame_len
    frames = 96
    G = np.ascontiguousarray(np.concatenate([np.eye(code.k, dtype=np.uint8), codes.gf2_parity_matrix(code)], 1))
    pipe = RxPipeline(t, code.n, code.k, blocks, 1e-3, max_batch_frames=frames)
    pipe.upload_tx_tables(generator_kn=G)
    rng = np.random.default_rng(700 + rank)
    info = torch.from_numpy(rng.integers(0, 2, size=(frames, blocks * code.k), dtype=np.uint8)).cuda()
    d_fr = torch.empty((frames, fl), dtype=torch.complex64, device="cuda")
    pipe.tx_batch(info, frames, d_fr, stream=torch.cuda.current_stream())
    tx = d_fr.cpu().numpy()
    # back-to-back frames with gaps inside the tracking window, AWGN and a 0.05-subcarrier offset
    gaps = rng.integers(0, 200, size=frames)
    x = np.concatenate([np.concatenate([tx[f], np.zeros(gaps[f], np.complex64)]) for f in range(frames)])
    n = np.arange(x.size)
    x = (x * np.exp(2j * np.pi * 0.05 / t.cfg.nfft * n)).astype(np.complex64)
    x += (1e-3 * (rng.standard_normal(x.size) + 1j * rng.standard_normal(x.size))).astype(np.complex64)
    host = torch.empty(x.size, dtype=torch.complex64, pin_memory=True)
    host.numpy()[:] = x
    block = 16384
    reps = max(args.steps, 1)

    def run_once():
        ing = Ingest(pipe, ring_samples=1 << 20, pool_frames=64)
        found = 0
        for at in range(0, x.size, block):
            ing.push(host[at: at + block])
            for slot, _, _, _ in ing.step(timeout_ms=0):
                ing.release(slot)
                found += 1
        st = ing.stats()
        ing.close()
        return found, st

    for _ in range(args.warmup):
        run_once()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    for _ in range(reps):
        found, st = run_once()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    value = world * reps * x.size / wall / 1e6
    line = {"metric": "Msample/s real-time ingest (device ring push + frame extraction), OFDM 16-QAM PHY",
            "value": round(value, 3), "unit": "Msample/s", "n_gpus": world, "steps": reps, "warmup": args.warmup,
            "ms_per_step": round(wall / reps * 1e3, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (GPU-transmitted frames, AWGN, CFO)",
            "config": {"workload": "ofdm_ingest_1024_512", "frames": frames, "samples": int(x.size),
                       "push_block": block, "ring_samples": 1 << 20, "pool_frames": 64,
                       "real_time_msps": t.cfg.sample_rate / 1e6},
            "frames_found": found, "stats": {k: int(v) for k, v in st.items()},
            "x_real_time": round(value / (t.cfg.sample_rate / 1e6), 2),
            "gpu_launches": int(reps * np.ceil(x.size / block)), "clocks": clk, "roofline": None,
            "e2e": {"value": round(value, 3), "unit": "Msample/s", "h2d_bytes_per_step": int(x.size * 8),
                    "d2h_bytes_per_step": int(found * 16)},
            "cpu_baseline": None}
    return line if rank == 0 else None


# --------------------------------------------------- mixed-code batched workload
def run_mixed(args, rank, world):
    """100,000 codewords of 15 codes in one persistent launch, against one launch per request."""
    import torch
    from sicc_gb300 import engine, fec

    dev = int(os.environ.get("LOCAL_RANK", 0))
    # CPU baseline pool: spawned before the first GPU call of this process
    pool = workers = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        workers = os.cpu_count() or 1
        pool = mp.get_context("spawn").Pool(workers)
    torch.cuda.set_device(dev)
    w = engine.mixed_workload(total=args.mixed_codewords, seed=4242 + rank)
    stream = torch.cuda.current_stream()
    d_code = torch.from_numpy(w.code_of).cuda()
    d_llr = torch.from_numpy(w.llr).cuda()
    d_llr_off = torch.from_numpy(w.llr_off).cuda()
    d_info_off = torch.from_numpy(w.info_off).cuda()
    d_info = torch.zeros(w.info_bits, dtype=torch.uint8, device="cuda")
    d_ok = torch.zeros(w.count, dtype=torch.uint8, device="cuda")
    d_used = torch.zeros(w.count, dtype=torch.uint8, device="cuda")
    d_it = torch.zeros(w.count, dtype=torch.uint8, device="cuda")
    eng = engine.Engine(max_codewords=w.count, max_llr_floats=w.llr.size)
    for c in w.codes:  # OSD order 2 for n <= 256, order 1 for the longer codes
        eng.add_code(c, engine.iteration_cap(c.n), ALPHA, 0.0, engine.osd_order_for(c), OSD_FLIP, OSD_TESTS)

    tuned = None
    if not args.no_tune:  # warps per codeword of each code and warps per CTA, on this batch
        base_ms, tuned_ms = eng.autotune(w.count, d_code, d_llr, d_llr_off, d_info, d_info_off, reps=2)
        tuned = {"bp_default_ms": round(base_ms, 4), "bp_tuned_ms": round(tuned_ms, 4)}
    code_warps = {c.name(): eng.code_warps(i) for i, c in enumerate(w.codes)}

    def batched():
        eng.decode_device(w.count, d_code, d_llr, d_llr_off, d_info, d_info_off, d_ok, d_used, d_it, stream=stream)

    for _ in range(args.warmup):
        batched()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        batched()
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    prep_ms, bp_ms, osd_ms = eng.last_ms()
    value = world * w.info_bits * args.steps / (elapsed_ms * 1e-3) / 1e6
    info = d_info.cpu().numpy()
    fe = np.zeros(w.count, bool)
    for i in range(0, w.count):
        a, k = w.info_off[i], w.codes[w.code_of[i]].k
        fe[i] = not np.array_equal(info[a:a + k], w.info_true[a:a + k])
    fer_by_n = {}
    for n in sorted({c.n for c in w.codes}):
        sel = np.array([w.codes[c].n == n for c in w.code_of])
        fer_by_n[str(n)] = float(fe[sel].mean())

    # plain form, as the reference decodes a frame (uhd_ldpc_ofdm_link.cpp:3541-3628, 3744-3785): one
    # decoder per code, one synchronous call per request with device LLRs in and host outputs.  Codes
    # beyond the reference decoder's OSD limits (n <= 256, k <= 128) run BP + OSD through a one-code
    # engine per request, so both forms do the same work.
    class OneCodeEngine:
        def __init__(self, c):
            self.c = c
            self.eng = engine.Engine(max_codewords=512, max_llr_floats=512 * c.n, max_codes=1)
            self.eng.add_code(c, engine.iteration_cap(c.n), ALPHA, 0.0, engine.osd_order_for(c), OSD_FLIP, OSD_TESTS)
            self.ids = torch.zeros(512, dtype=torch.uint8, device="cuda")
            self.lo = torch.arange(512, dtype=torch.int64, device="cuda") * c.n
            self.io = torch.arange(512, dtype=torch.int64, device="cuda") * c.k
            self.info = torch.zeros(512 * c.k, dtype=torch.uint8, device="cuda")
            self.ok = torch.zeros(512, dtype=torch.uint8, device="cuda")

        def decode(self, llr_v, device=True):
            b = llr_v.shape[0]
            self.eng.decode_device(b, self.ids, llr_v, self.lo, self.info, self.io, self.ok, stream=stream)
            return self.info[: b * self.c.k].cpu().numpy(), self.ok[:b].cpu().numpy()

    decs = []
    for c in w.codes:
        if engine.osd_supported(c):
            decs.append(fec.StreamBpOsdDecoder(c, max_batch=512, min_batch=1, max_iter=engine.iteration_cap(c.n),
                                               normalization=ALPHA, offset=0.0, damping=0.0, min_abs_llr_accept=0.0,
                                               osd_order=OSD_ORDER, osd_max_flip=OSD_FLIP, osd_max_tests=OSD_TESTS))
        else:
            decs.append(OneCodeEngine(c))

    def plain_pass():
        for r, ci in enumerate(w.req_code):
            a, b = int(w.req_start[r]), int(w.req_start[r + 1])
            n = w.codes[ci].n
            llr_v = d_llr[int(w.llr_off[a]): int(w.llr_off[a]) + (b - a) * n].view(b - a, n)
            decs[ci].decode(llr_v, device=True)  # submit + flush + poll / device-batch call, host outputs

    plain_pass()
    t0 = time.perf_counter()
    plain_pass()
    plain_s = time.perf_counter() - t0
    plain_mbps = w.info_bits / plain_s / 1e6

    # end to end: pinned host LLRs in, host information bits out, every step on the decode stream
    e2e = None
    if not args.no_e2e:
        h_llr = torch.empty(w.llr.shape, dtype=torch.float32, pin_memory=True)
        h_llr.numpy()[:] = w.llr
        h_info = torch.empty(w.info_bits, dtype=torch.uint8, pin_memory=True)

        def e2e_step():
            d_llr.copy_(h_llr, non_blocking=True)
            batched()
            h_info.copy_(d_info, non_blocking=True)

        e2e_step()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        torch.cuda.synchronize()
        e2e_s = time.perf_counter() - t0
        e2e = {"value": round(world * w.info_bits * args.steps / e2e_s / 1e6, 3), "unit": "Mbit/s",
               "h2d_bytes_per_step": int(w.llr.nbytes), "d2h_bytes_per_step": int(w.info_bits),
               "api": "sicc_engine_decode_device between pinned-host copies on the same stream"}

    cpu = None
    if pool is not None:  # every code's first requests, up to 256 codewords per code, on all host cores
        tasks, bits = [], 0
        for ci, c in enumerate(w.codes):
            rows = [i for i in range(w.count) if w.code_of[i] == ci][:256]
            if not rows:
                continue
            llr = np.stack([w.llr[w.llr_off[i]: w.llr_off[i] + c.n] for i in rows])
            for part in np.array_split(llr, max(1, min(len(rows), workers // len(w.codes) + 1))):
                if len(part):
                    tasks.append((c.n, c.m, c.row_ptr, c.col_ind, part, engine.iteration_cap(c.n),
                                  engine.osd_order_for(c)))
            bits += len(rows) * c.k
        c0 = time.perf_counter()
        pool.map(_cpu_mixed_worker, tasks)
        cs = time.perf_counter() - c0
        cpu = {"value": round(bits / cs / 1e6, 4), "unit": "Mbit/s", "cores": workers, "kind": "port",
               "sample": f"up to 256 codewords of each of the 15 codes ({bits} information bits): the restated "
                         "row-sequential layered min-sum + generator OSD (oracle/sicc_oracle.c)"}
        pool.close()
    peak, peak_kind = peaks()
    line = {"metric": "info-bit Mbps mixed-code BP(+OSD), 100k codewords, 15 codes", "value": round(value, 3),
            "unit": "Mbit/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded BPSK/AWGN LLRs, Eb/N0 ~ U[1,5] dB)",
            "config": {"workload": "mixed_100k", "codewords": w.count, "requests": int(len(w.req_code)),
                       "lengths": [128, 256, 512, 1024, 2048], "rates": ["1/2", "11/16", "3/4"],
                       "bp": "layered NMS alpha 0.75, 20/25/30 iterations by length",
                       "osd": "on failing codewords: order 2 (n <= 256), order 1 (n >= 512)",
                       "l2": f"{w.llr.nbytes / 1e6:.0f} MB of LLRs per step (> L2)",
                       "warps_per_codeword": code_warps, "autotune": tuned},
            "fer_by_length": fer_by_n, "fer": float(fe.mean()),
            "kernel_ms": {"prepare": round(prep_ms, 4), "bp_mixed": round(bp_ms, 4), "osd": round(osd_ms, 4)},
            "plain_one_code_per_launch": {"value": round(plain_mbps, 3), "unit": "Mbit/s",
                                          "calls_per_pass": int(len(w.req_code)),
                                          "api": "per request: cuda_osd_submit_device_codewords+flush+poll_ready "
                                                 "(n <= 256, k <= 128) or a one-code engine call; host outputs, "
                                                 "synchronous",
                                          "speedup_of_batched": round(value / plain_mbps, 2)},
            "gpu_launches": args.steps * 3, "clocks": clk,
            "roofline": {"bound": "hbm", "kernel": "bp_mixed_kernel<16>",
                         "achieved": round((w.llr.nbytes + w.info_bits) / (bp_ms * 1e-3) / 1e9, 2), "peak": peak,
                         "unit": "GB/s",
                         "frac": round((w.llr.nbytes + w.info_bits) / (bp_ms * 1e-3) / 1e9 / peak, 5),
                         "traffic": traffic_for("bp_mixed_kernel<16>", w.count), "peak_source": peak_kind,
                         "note": "issue-bound; HBM fraction shown per contract"},
            "e2e": e2e, "cpu_baseline": cpu}
    return line if rank == 0 else None


# ------------------------------------------------------------ long-code workload
DVBS2_PROFILE, DVBS2_EBN0, DVBS2_ITERS, DVBS2_FRAMES = "N64800_R1/2", 2.0, 30, 1216


def run_dvbs2(args, rank, world):
    """Colored-layered BP of a DVB-S2-sized (64800,32400) IRA code through the CSR BP decoder."""
    import torch
    from sicc_gb300 import channel, codes, fec

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    code = codes.dvbs2_code(args.dvbs2_profile)
    frames = args.dvbs2_frames
    resident = 2  # 2 x 315 MB of LLRs cycled (> L2) at 1216 frames
    data = [channel.awgn_llrs(code, frames, DVBS2_EBN0, seed=3000 + 10 * rank + i) for i in range(resident)]
    d_llr = [torch.from_numpy(x[2]).cuda() for x in data]
    d_bits = torch.empty((frames, code.n), dtype=torch.uint8, device="cuda")
    d_ok = torch.empty(frames, dtype=torch.uint8, device="cuda")
    d_it = torch.empty(frames, dtype=torch.uint8, device="cuda")
    dec = fec.CsrBpDecoder(code.n, code.m, code.row_ptr, code.col_ind, max_batch=frames, max_iter=DVBS2_ITERS,
                           normalization=ALPHA, schedule=fec.COLORED_LAYERED)
    stream = torch.cuda.current_stream()

    def step(s):
        dec.decode_device_batch(d_llr[s % resident], d_bits, d_ok, None, d_it, stream=stream)

    for s in range(args.warmup):
        step(s)
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for s in range(args.steps):
        step(s)
    ev1.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    elapsed_ms = ev0.elapsed_time(ev1)
    value = world * frames * code.k * args.steps / (elapsed_ms * 1e-3) / 1e6
    step(0)
    torch.cuda.synchronize()
    ok = d_ok.cpu().numpy().astype(bool)
    bits = d_bits.cpu().numpy()
    fer = float(np.mean(~ok | np.any(bits[:, : code.k] != data[0][0], axis=1)))
    iters = float(d_it.cpu().numpy().mean())

    # end to end: the host entry point (cuda_osd_decode_bp_csr_batch) with pinned host LLRs
    e2e = None
    if not args.no_e2e:
        h_llr = torch.empty((frames, code.n), dtype=torch.float32, pin_memory=True)
        h_llr.numpy()[:] = data[0][2]
        dec.decode(h_llr.numpy())
        t0 = time.perf_counter()
        for _ in range(args.steps):
            dec.decode(h_llr.numpy())
        e2e_s = time.perf_counter() - t0
        e2e = {"value": round(world * frames * code.k * args.steps / e2e_s / 1e6, 3), "unit": "Mbit/s",
               "h2d_bytes_per_step": frames * code.n * 4, "d2h_bytes_per_step": frames * (code.n + 1),
               "api": "cuda_osd_decode_bp_csr_batch (pinned host LLRs in, host code bits out)"}

    cpu = None
    if not args.no_cpu_baseline and rank == 0:  # the restated layered decoder on one host core
        from oracle import Oracle, build_oracle
        build_oracle()
        oc = Oracle().code(code.n, code.m, code.row_ptr, code.col_ind)
        order, _, _ = oc.color_order()
        sample = 8
        c0 = time.perf_counter()
        for x in data[1][2][:sample]:
            oc.layered(x, DVBS2_ITERS, ALPHA, row_order=order)
        cs = time.perf_counter() - c0
        cpu = {"value": round(sample * code.k / cs / 1e6, 4), "unit": "Mbit/s", "cores": 1, "kind": "port",
               "sample": f"{sample} codewords, colored-layered min-sum (oracle/sicc_oracle.c), one core"}

    peak, peak_kind = peaks()
    algo = frames * (4 * code.n + code.n + 2)  # LLRs in; code bits, success, iterations out
    achieved = algo / (elapsed_ms / args.steps * 1e-3) / 1e9
    line = {"metric": "info-bit Mbps BP, long IRA code (DVB-S2 size), colored-layered min-sum",
            "value": round(value, 3), "unit": "Mbit/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(elapsed_ms / args.steps, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded BPSK/AWGN LLRs, seeded IRA address tables)",
            "config": {"workload": "dvbs2_64800_r12" if args.dvbs2_profile == DVBS2_PROFILE else
                       "dvbs2_" + args.dvbs2_profile.lower().replace("/", ""),
                       "code": f"IRA ({code.n},{code.k}), DVB-S2 {args.dvbs2_profile} "
                                                                  "degree profile",
                       "ebn0_db": DVBS2_EBN0, "max_iter": DVBS2_ITERS, "alpha": ALPHA, "schedule": "colored layered",
                       "frames_per_step": frames, "l2": f"2 resident batches of {frames * code.n * 4 / 1e6:.0f} MB cycled"},
            "fer": fer, "mean_iterations": round(iters, 3), "gpu_launches": args.steps,
            "clocks": clk,
            "roofline": {"bound": "hbm", "kernel": "bp_layered_wide_kernel<8>", "achieved": round(achieved, 2),
                         "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 5), "traffic": None,
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": algo,
                         "note": "decoder state is L2-resident per CTA; the kernel is latency-bound, HBM fraction "
                                 "shown per contract"},
            "e2e": e2e, "cpu_baseline": cpu}
    return line if rank == 0 else None


# ------------------------------------------------------------------ serving loop
SERVE_LOADS = (0.1, 0.3, 0.5, 0.7, 0.8, 0.9, 1.0, 1.2)


def run_serve(args, rank, world):
    """Poisson arrivals of decode requests into the continuous-batching server.

    Requests: bursts of U{1..512} codewords of one of the 15 mixed codes (Eb/N0 ~ U[1,5] dB per codeword),
    or, with probability 0.3, U{1..17} frames of the 16-QAM OFDM workload (up to 510 codewords of the
    (1024,512) code) as raw IQ that the server demodulates first.  Protection per request: BP only or
    BP+OSD with probability 1/2 (OSD where the code has OSD tables: n <= 256, k <= 128).  The peak is the
    throughput with every request offered at once; the sweep offers Poisson load at fractions of it.
    Inputs and outputs live in pinned host memory; latency runs from the scheduled arrival to the results
    on the host.
    """
    import torch
    from sicc_gb300 import channel, codes, engine, ofdm
    from sicc_gb300.server import Server

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    rng = np.random.default_rng(777 + rank)
    mixed = codes.mixed_codes()
    ocode = codes.ofdm_code()
    t = ofdm.reference_tables(ofdm.OFDM_C3)
    blocks = t.coded_bits // ocode.n

    def pinned(shape, dtype):
        return torch.empty(shape, dtype=dtype, pin_memory=True).numpy()

    # request pools (pinned): 512 codewords per code, 24 frames per SNR point
    llr_pool, info_pool = [], []
    for ci, c in enumerate(mixed):
        info, _, llr = channel.awgn_llrs(c, 512, rng.uniform(1.0, 5.0, 512), seed=9000 + ci)
        buf = pinned((512, c.n), torch.float32)
        buf[:] = llr
        llr_pool.append(buf)
        info_pool.append(info)
    iq_pool, iq_info = [], []
    for i, snr in enumerate(OFDM_SNRS):
        gen = ofdm.FrameGenerator(t, ocode, seed=600 + i)
        b = gen.batch(24, snr_db=snr, cfo_subcarriers=0.1, max_offset=200, rayleigh_taps=6)
        buf = pinned(b.iq.shape, torch.complex64)
        buf[:] = b.iq
        iq_pool.append((buf, float(np.float32(np.mean(b.noise_var)))))
        iq_info.append(b.info)
    stride = iq_pool[0][0].shape[1]

    device_loop = getattr(args, "serve_loop", "host") == "device"
    if device_loop:
        # the device-resident loop: loop_lanes lanes (batches decoded side by side), one lane iteration
        # holds up to loop_batch codewords (their LLRs: up to 2048 floats each) and 17 x 16 frames of IQ
        from sicc_gb300.devloop import DevLoop
        srv = DevLoop(max_batch_codewords=args.loop_batch, max_batch_llr_floats=args.loop_batch * 2048,
                      ring_requests=4096, idle_timeout_ms=2000, max_batch_frames=272,
                      max_batch_iq_samples=272 * stride, lanes=args.loop_lanes)
    else:
        srv = Server(hbm_budget_bytes=40 << 30, max_batch_codewords=args.serve_batch,
                     max_inflight_batches=args.serve_inflight, max_pending_requests=1 << 16)
    ids = [srv.add_code(c, engine.iteration_cap(c.n), ALPHA, engine.osd_order_for(c),
                        OSD_FLIP, OSD_TESTS) for c in mixed]
    ocid = srv.add_code(ocode, OFDM_ITERS, ALPHA, engine.osd_order_for(ocode))
    phys = [srv.add_phy(t, ocid, blocks, nv, stride) for _, nv in iq_pool]
    srv.start()

    def make_request(kind, ident, data, prot, tag, out):
        if not device_loop:
            return srv.request(kind, ident, data, prot, tag=tag, out=out)
        if kind == 1:
            return srv.iq_request(ident, data, prot, tag=tag, out=out)
        return srv.request(ident, data, prot, tag=tag, out=out)

    # one request list, reused at every load point (outputs are overwritten)
    n_req = args.serve_requests
    reqs, truth, info_bits, iq_reqs = [], [], 0, 0
    for r in range(n_req):
        prot = int(rng.integers(0, 2))
        if rng.random() < 0.3:
            s = int(rng.integers(0, len(OFDM_SNRS)))
            f = int(rng.integers(1, 18))
            a = int(rng.integers(0, 24 - f + 1))
            out = pinned((f * blocks, ocode.k), torch.uint8)
            reqs.append(make_request(1, phys[s], iq_pool[s][0][a:a + f], prot, r, out))
            truth.append(iq_info[s][a:a + f].reshape(f * blocks, ocode.k))
            info_bits += f * blocks * ocode.k
            iq_reqs += 1
        else:
            ci = int(rng.integers(0, len(mixed)))
            b = int(rng.integers(1, 513))
            a = int(rng.integers(0, 512 - b + 1))
            out = pinned((b, mixed[ci].k), torch.uint8)
            reqs.append(make_request(0, ids[ci], llr_pool[ci][a:a + b], prot, r, out))
            truth.append(info_pool[ci][a:a + b])
            info_bits += b * mixed[ci].k
    in_bytes = sum(int(q[1].nbytes) for q in reqs)
    out_bytes = sum(int(q[2].nbytes) for q in reqs)
    at_once = np.zeros(n_req)
    is_iq = np.array([q[0].kind == 1 for q in reqs])
    bp_only = np.array([q[0].protection == 0 for q in reqs])

    def progress(msg):
        print(f"[serve] {msg}", file=sys.stderr, flush=True)

    progress(f"{n_req} requests, {info_bits} info bits; warm-up")
    for _ in range(args.warmup):
        _, wall = srv.replay(reqs, at_once)
        progress(f"warm-up replay {wall * 1e-6:.3f} s")
    clocks = ClockSampler(dev)
    clocks.start()
    time.sleep(0.3)
    st0 = srv.stats()
    walls = []
    for _ in range(args.steps):
        res, wall = srv.replay(reqs, at_once)
        walls.append(wall)
    st1 = srv.stats()
    peak_s = statistics.median(walls) * 1e-6
    peak_mbps = info_bits / peak_s / 1e6
    progress(f"peak {peak_mbps:.1f} Mbit/s ({peak_s:.3f} s per pass)")
    fe = [int(np.any(q[2] != tr, axis=1).sum()) for q, tr in zip(reqs, truth)]
    cw_total = sum(q[2].shape[0] for q in reqs)
    sweep = []
    for load in (args.serve_loads or SERVE_LOADS):
        rate = load * n_req / peak_s  # requests per second
        gaps = rng.exponential(1.0 / rate, n_req)
        arr = np.cumsum(gaps) * 1e6
        arr -= arr[0]
        b0 = srv.stats()
        res, wall = srv.replay(reqs, arr)
        b1 = srv.stats()
        progress(f"load {load}: {wall * 1e-6:.3f} s")
        lat = np.array([d.latency_us for d in res]) * 1e-3
        wait = np.array([d.launch_us for d in res]) * 1e-3
        gpu = np.array([d.batch_gpu_us for d in res]) * 1e-3
        sweep.append({"load": load, "offered_mbps": round(load * peak_mbps, 2),
                      "achieved_mbps": round(info_bits / (wall * 1e-6) / 1e6, 2),
                      "p50_ms": round(float(np.percentile(lat, 50)), 4),
                      "p99_ms": round(float(np.percentile(lat, 99)), 4),
                      "p99_9_ms": round(float(np.percentile(lat, 99.9)), 4),
                      "p99_ms_llr_requests": round(float(np.percentile(lat[~is_iq], 99)), 4),
                      "p99_ms_iq_requests": round(float(np.percentile(lat[is_iq], 99)), 4),
                      "p50_ms_bp_only": round(float(np.percentile(lat[bp_only], 50)), 4),
                      "p99_ms_bp_only": round(float(np.percentile(lat[bp_only], 99)), 4),
                      "p99_ms_bp_osd": round(float(np.percentile(lat[~bp_only], 99)), 4),
                      "p50_wait_ms": round(float(np.percentile(wait, 50)), 4),
                      "p50_batch_gpu_ms": round(float(np.percentile(gpu, 50)), 4),
                      "p99_batch_gpu_ms": round(float(np.percentile(gpu, 99)), 4),
                      "mean_batch_codewords": round((b1.codewords - b0.codewords) /
                                                    max(_batches(b1) - _batches(b0), 1), 1),
                      "batches": int(_batches(b1) - _batches(b0))})
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    p80 = next((x for x in sweep if x["load"] == 0.8), sweep[-1])
    if device_loop:
        # every loop iteration: admit, publish; one that admitted requests also: layout, sync + demod per
        # profile, prepare, mixed BP, the OSD launches (warp kernel and three long-code classes), complete
        launches = (int(st1.iterations - st0.iterations) * 2
                    + int(_batches(st1) - _batches(st0)) * (2 + 2 * len(phys) + 2 + 4))
    else:
        launches = int(st1.batches - st0.batches) * 3 + args.steps * iq_reqs * 2
    line = {"metric": "served info-bit Mbps (Poisson mixed-code + OFDM IQ requests), p50/p99/p99.9 latency",
            "value": round(peak_mbps, 3), "unit": "Mbit/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(peak_s * 1e3, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded BPSK/AWGN LLRs; seeded OFDM IQ: 6-tap Rayleigh, CFO 0.1 sc, SNR 8/12/16 dB)",
            "config": {"workload": "serve_mixed", "requests": n_req, "iq_requests": iq_reqs,
                       "codewords": cw_total, "info_bits": info_bits, "hbm_budget_gb": 40,
                       "max_batch_codewords": args.loop_batch if device_loop else args.serve_batch,
                       "inflight_batches": args.loop_lanes if device_loop else args.serve_inflight,
                       "burst": "U{1..512} codewords or U{1..17} OFDM frames (p=0.3)",
                       "protection": "BP or BP+OSD (p=1/2); OSD order 2 (n <= 256), order 1 (n >= 512)",
                       "step": "every request offered at once (peak); then one Poisson pass per load point",
                       "l2": "inputs copied host->device every request (pinned host pools)"},
            "fer": round(sum(fe) / cw_total, 5), "load_sweep": sweep,
            "p99_ms_at_80pct_load": p80["p99_ms"],
            "server": ({"loop": "device-resident (conditional CUDA graphs sharing the rings; include/sicc_devloop.h)",
                        "lanes": int(st.lanes), "iterations": int(st.iterations),
                        "busy_iterations": int(st.busy_iterations), "graph_launches": int(st.launches),
                        "busy_rejections": int(st.busy_rejections)} if device_loop else
                       {"loop": "host scheduler thread (include/sicc_server.h)", "batches": int(st.batches),
                        "busy_rejections": int(st.busy_rejections),
                        "arena_peak_mb": round(st.arena_bytes_peak / 1e6, 1)}),
            "gpu_launches": launches, "clocks": clk, "roofline": None,
            "e2e": {"value": round(peak_mbps, 3), "unit": "Mbit/s", "h2d_bytes_per_step": in_bytes,
                    "d2h_bytes_per_step": out_bytes},
            "cpu_baseline": None}
    return line if rank == 0 else None


# ------------------------------------- per-frame Pipeline class (reference benchmark configuration)
FRAME_BENCH_SRC = os.path.join(ROOT, "tests", "cpp", "ofdm_frame_bench.cpp")


def _frame_bench_line(impl, res, wall_s, frames, clk, extra):
    """JSON line of the per-frame Pipeline workload from the benchmark program's output."""
    mbps = res["rx_fps"] * res["info_bits_per_frame"] / 1e6
    line = {"metric": "frames/s through Pipeline::demod_frame_to_host_llr (host frame -> sync + demod -> host LLRs), "
                      "reference GPU pipeline benchmark configuration",
            "value": round(res["rx_fps"], 2), "unit": "frames/s", "n_gpus": 1, "steps": frames, "warmup": 64,
            "ms_per_step": round(1e3 / res["rx_fps"], 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (noiseless QPSK OFDM loop-back frames)",
            "config": {"workload": "ofdm_frame_pipeline", "fft": 1024, "cp": 72, "symbols": 96, "pilot_period": 4,
                       "active_sc": 768, "modulation": "QPSK", "pre_half_len": 256,
                       "frame_samples": res["frame_samples"], "coded_bits_per_frame": res["coded_bits_per_frame"],
                       "code": "repetition (128,64)", "slots": 3,
                       "source": "gpu_ofdm_pipeline_bench.cpp:21-38 defaults"},
            "rx_info_mbps": round(mbps, 2), "tx_fps": round(res["tx_fps"], 2),
            "roundtrip_fps": round(res["roundtrip_fps"], 2),
            "hard_check": {"bits": res["checked_bits"], "errors": res["hard_errors"]},
            "clocks": clk, "e2e": {"value": round(res["rx_fps"], 2), "unit": "frames/s",
                                   "h2d_bytes_per_step": res["frame_samples"] * 8,
                                   "d2h_bytes_per_step": res["coded_bits_per_frame"] * 4}}
    if impl == "reference":
        line["impl"] = "reference"
    line.update(extra)
    return line


def _run_frame_bench(exe, frames):
    out = subprocess.run([exe, "--frames", str(frames), "--warmup", "64"], capture_output=True, text=True,
                         timeout=900)
    if out.returncode != 0:
        raise RuntimeError(f"{os.path.basename(exe)} exited {out.returncode}: {out.stderr[-500:]}")
    return json.loads([ln for ln in out.stdout.splitlines() if ln.startswith("{")][-1])


def run_frame_pipeline(args, rank, world):
    """The per-frame Pipeline class path, timed by one driver (tests/cpp/ofdm_frame_bench.cpp) built
    against this library; the reference arm builds the same driver against the reference's pipeline."""
    if rank != 0:
        return None
    from sicc_gb300 import _lib
    if not os.path.exists(_lib.LIB_PATH):
        raise RuntimeError(f"{_lib.LIB_PATH} is missing: run __graft_entry__.build() first")
    libdir = os.path.dirname(_lib.LIB_PATH)
    os.makedirs(os.path.join(ROOT, "_build"), exist_ok=True)
    exe = os.path.join(ROOT, "_build", "ofdm_frame_bench_gb300")
    subprocess.run(["g++", "-O3", "-std=c++17", "-I" + os.path.join(ROOT, "include"), FRAME_BENCH_SRC, "-o", exe,
                    "-L" + libdir, "-lsicc_gb300", "-Wl,-rpath," + libdir], check=True)
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    t0 = time.perf_counter()
    res = _run_frame_bench(exe, args.frame_bench_frames)
    wall = time.perf_counter() - t0
    clk = clocks.stop()
    return _frame_bench_line("ours", res, wall, args.frame_bench_frames, clk,
                             {"gpu_launches": args.frame_bench_frames * 2,  # the timed receive loop
                              "kernels_per_rx_frame": ["sync_kernel", "demod_kernel"],
                              "cpu_baseline": None, "roofline": None})


def run_frame_pipeline_reference(args, rank, world):
    """Reference arm of the per-frame workload: the same driver linked with the reference's own CUDA
    pipeline (gpu_ofdm_pipeline.cu, staged under oracle/_ref/src), plus the reference's unmodified
    benchmark program for comparison."""
    if rank != 0:
        return None
    stage = os.path.join(ROOT, "oracle", "_ref", "src", "pipeline", "gpu_ofdm_pipeline.cu")
    if not os.path.exists(stage):
        return {"impl": "reference", "unavailable": "the reference's GPU pipeline sources were not staged "
                                                    "(make -C oracle stage where the reference tree is present)"}
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ofdm-bench"], check=True)
    exe = os.path.join(ROOT, "oracle", "_ref", "ofdm_frame_bench_ref")
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", 0)))
    clocks.start()
    res = _run_frame_bench(exe, args.frame_bench_frames)
    clk = clocks.stop()
    own = subprocess.run([os.path.join(ROOT, "oracle", "_ref", "gpu_ofdm_pipeline_bench_ref"), "--frames",
                          str(args.frame_bench_frames)], capture_output=True, text=True, timeout=900)
    own_lines = [ln for ln in own.stdout.splitlines() if ln.startswith("[GPU-BENCH]")]
    return _frame_bench_line("reference", res, 0.0, args.frame_bench_frames, clk,
                             {"gpu_launches": 0, "cpu_baseline": None, "roofline": None,
                              "reference_own_benchmark": {"rc": own.returncode, "output": own_lines}})


def _batches(st):
    """Batches launched by the host-scheduled server, or device-loop iterations that admitted requests."""
    return st.batches if hasattr(st, "batches") else st.busy_iterations


# ------------------------------------------------------------- reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return
    workers = os.cpu_count() or 1
    pool = mp.get_context("spawn").Pool(workers)
    # the same frames as the GPU arm's first resident batch (rank 0's seeds), first cpu_sample of each
    code, inputs = make_inputs(BATCH, 1, seed0=1000)
    sample = {e: (inputs[e][0][0][: args.cpu_sample], inputs[e][0][2][: args.cpu_sample]) for e in EBN0}
    for _ in range(max(1, min(args.warmup, 1))):  # also builds each worker's code tables
        cpu_decode(pool, workers, sample[EBN0[0]][1][: workers * 32])
    wall = 0.0
    fer = {}
    for s in range(args.steps):
        for e in EBN0:
            w, info, _ = cpu_decode(pool, workers, sample[e][1])
            wall += w
            if s == 0:
                fer[f"{e:g}dB"] = float(np.mean(np.any(info != sample[e][0], axis=1)))
    pool.close()
    bits = args.steps * len(EBN0) * args.cpu_sample * code.k
    value = bits / wall / 1e6
    sample = (f"the first {args.cpu_sample} frames of the GPU arm's first batch at each of 2 and 3 dB, every step: "
              f"the reference decoder (flooding min-sum alpha 0.75, 20 iterations, order-2 OSD on the "
              f"best-syndrome posterior), {workers} worker processes")
    line = {"impl": "reference", "metric": "info-bit Mbps BP+OSD (128,64), Eb/N0 2 and 3 dB",
            "value": round(value, 4), "unit": "Mbit/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(wall * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded BPSK/AWGN LLRs)",
            "config": {"workload": WORKLOAD, "code": "QC (128,64) 4x8 base Z=16", "ebn0_db": list(EBN0),
                       "frames_per_step": len(EBN0) * args.cpu_sample, "parallelism": "host cores"},
            "fer": fer, "gpu_launches": 0,
            "cpu_baseline": {"value": round(value, 4), "unit": "Mbit/s", "cores": workers, "kind": "port",
                             "sample": sample},
            "e2e": {"value": round(value, 4), "unit": "Mbit/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    return line


def run_targets(args):
    """Short runs of the two systems targets, reported beside the headline (1 GPU, same process).

    * Mixed-code batching (100,000 codewords of 15 codes): one persistent batched launch against the
      plain form, one synchronous decode call per request; target: batched >= 50x plain.
    * Serving: every request offered at once gives the peak, then one Poisson pass at 80% of it;
      target: p99 request latency < 1 ms at 80% load.  Run twice: through the host-scheduled server
      and through the device-resident graph loop.
    """
    import copy
    sub = copy.copy(args)
    sub.steps, sub.warmup, sub.no_e2e, sub.no_cpu_baseline = 5, 3, True, True
    mixed = run_mixed(sub, 0, 1)
    sub = copy.copy(args)
    sub.steps, sub.warmup, sub.no_e2e, sub.no_cpu_baseline = 3, 1, True, True
    sub.serve_loads = (0.8,)
    serve = run_serve(sub, 0, 1)
    sub.serve_loop = "device"
    serve_dev = run_serve(sub, 0, 1)
    plain = mixed["plain_one_code_per_launch"]
    p80 = serve["load_sweep"][0]
    return {"mixed_batched_vs_plain": {"batched_mbps": mixed["value"], "plain_mbps": plain["value"],
                                       "ratio": plain["speedup_of_batched"], "target_ratio": 50,
                                       "kernel_ms": mixed["kernel_ms"], "fer": mixed["fer"],
                                       "workload": "mixed_100k (5 timed steps)"},
            "serving_p99_at_80pct": {"peak_mbps": serve["value"], "offered_mbps": p80["offered_mbps"],
                                     "achieved_mbps": p80["achieved_mbps"], "p50_ms": p80["p50_ms"],
                                     "p99_ms": p80["p99_ms"], "p99_9_ms": p80["p99_9_ms"],
                                     "p99_ms_bp_only": p80["p99_ms_bp_only"], "p99_ms_bp_osd": p80["p99_ms_bp_osd"],
                                     "target_p99_ms": 1.0,
                                     "workload": f"serve_mixed, {serve['config']['requests']} requests, "
                                                 "host-scheduled server"},
            "serving_device_loop_p99_at_80pct": _p80_summary(serve_dev)}


def _p80_summary(serve):
    p80 = serve["load_sweep"][0]
    return {"peak_mbps": serve["value"], "offered_mbps": p80["offered_mbps"], "achieved_mbps": p80["achieved_mbps"],
            "p50_ms": p80["p50_ms"], "p99_ms": p80["p99_ms"], "p99_9_ms": p80["p99_9_ms"],
            "p99_ms_bp_only": p80["p99_ms_bp_only"], "p99_ms_bp_osd": p80["p99_ms_bp_osd"], "target_p99_ms": 1.0,
            "workload": f"serve_mixed, {serve['config']['requests']} requests, device-resident loop",
            "iterations": serve["server"].get("iterations")}


def spawn_ranks(n, argv):
    """Runs bench.py with `argv` as `n` ranks on this node (127.0.0.1 rendezvous); returns the exit code."""
    import socket
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)] + list(argv)
    return subprocess.call(cmd)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=4096)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-targets", action="store_true", help="default workload: skip the short C4/C5 target runs")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shapes (no autotuner)")
    ap.add_argument("--batch", type=int, default=BATCH, help="frames per batch (profiling runs only)")
    ap.add_argument("--resident", type=int, default=RESIDENT_BATCHES, help="resident batches per Eb/N0")
    ap.add_argument("--workload", default=WORKLOAD, choices=[WORKLOAD, "ofdm_rx_1024_512", "ofdm_tx_1024_512", "ofdm_ingest_1024_512",
                                                        "mixed_100k", "serve_mixed", "dvbs2_64800_r12",
                                                        "ofdm_frame_pipeline"])
    ap.add_argument("--frame-bench-frames", type=int, default=4000, help="frames per stage of ofdm_frame_pipeline")
    ap.add_argument("--serve-requests", type=int, default=1500)
    ap.add_argument("--serve-loads", type=float, nargs="*", default=None, help="offered loads (fractions of peak)")
    ap.add_argument("--serve-batch", type=int, default=16384, help="codewords per server launch")
    ap.add_argument("--serve-inflight", type=int, default=4, help="batches overlapping on the device")
    ap.add_argument("--loop-lanes", type=int, default=8, help="device-loop lanes (batches side by side)")
    ap.add_argument("--loop-batch", type=int, default=4096, help="codewords per device-loop lane iteration")
    ap.add_argument("--serve-loop", default="host", choices=["host", "device"],
                    help="serving loop: host scheduler thread, or the device-resident graph loop")
    ap.add_argument("--mixed-codewords", type=int, default=100_000)
    ap.add_argument("--ofdm-frames", type=int, default=OFDM_FRAMES)
    ap.add_argument("--dvbs2-frames", type=int, default=DVBS2_FRAMES, help="codewords per long-code step")
    ap.add_argument("--dvbs2-profile", default=DVBS2_PROFILE, choices=["N64800_R1/2", "N16200_R1/4", "N16200_R1/2",
                                                                       "N16200_R5/6"],
                    help="frame size and degree profile of the long-code workload")
    args = ap.parse_args()
    globals()["BATCH"] = args.batch
    globals()["RESIDENT_BATCHES"] = args.resident
    if args.gpus > 1 and "RANK" not in os.environ:
        # one process per GPU: run this command again under torch.distributed.run with N ranks
        sys.exit(spawn_ranks(args.gpus, sys.argv[1:]))
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    if world != args.gpus:
        sys.exit(f"bench.py: --gpus {args.gpus} but WORLD_SIZE={world}")
    if args.impl == "reference" and args.workload == "ofdm_frame_pipeline":
        line = run_frame_pipeline_reference(args, rank, world)
    elif args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.workload == "ofdm_frame_pipeline":
        line = run_frame_pipeline(args, rank, world)
    elif args.workload == "ofdm_rx_1024_512":
        line = run_ofdm(args, rank, world)
    elif args.workload == "ofdm_tx_1024_512":
        line = run_ofdm_tx(args, rank, world)
    elif args.workload == "ofdm_ingest_1024_512":
        line = run_ingest(args, rank, world)
    elif args.workload == "mixed_100k":
        line = run_mixed(args, rank, world)
    elif args.workload == "serve_mixed":
        line = run_serve(args, rank, world)
    elif args.workload == "dvbs2_64800_r12":
        line = run_dvbs2(args, rank, world)
    else:
        line = run_ours(args, rank, world)
        if line is not None and world == 1 and not args.no_targets:
            line["targets"] = run_targets(args)
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
