"""The reference's own CUDA pipeline (cuFFT) beside this library on the same seeded
tomograms, on one GPU: wall time per tomogram and RI error of both against the FP64
oracle.  COMPARISON INFRASTRUCTURE ONLY.

Needs the sources assembled by oracle/refcuda/assemble.py (oracle/_ref/refcuda/src)
and nvcc; builds oracle/_ref/refcuda/ref_pipeline with oracle/refcuda/Makefile, then
for each workload writes the holograms to a file, runs the binary (its wall clock
covers hologram upload -> RI volume back on the host, as the reference's job loop
does it), and times this library through its host-buffer entry point
(ctdm_reconstruct_u16: integer photon counts uploaded as 16-bit, volume downloaded,
one call at a time) and with the holograms resident in HBM.

    python oracle/refcuda/compare.py [--configs plain_small,wrap_heavy,plain_512] [--reps 3] [--out FILE]
    python oracle/refcuda/compare.py --qpib [--out FILE]   (QPI Algorithm B only)
    python oracle/refcuda/compare.py --fastuw [--out FILE] (FastUnwrapping only)
    python oracle/refcuda/compare.py --residues [--out FILE] (Goldstein residues only)
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(os.path.dirname(HERE), "_ref", "refcuda")
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

CONFIGS = {
    # name: (iterations, run Goldstein in the benchmarked form of this library)
    "plain_small": (10, False),
    "wrap_heavy": (20, True),
    "plain_512": (10, False),
}


def workload(name):
    """Seeded acquisitions with the benchmark configurations' shapes: 49 x 256^2 -> 256^3;
    121 x 1024^2 -> 256^2 windows -> 256^3 (RI 1.40, 10 um cell); 181 x 1024^2 on a cone
    at NA 1.2 -> 512^3 (the differentiable configuration's acquisition, plain method)."""
    from ctdm_gb300 import phantom
    if name == "plain_small":
        return phantom.config_plain_small(seed=1000)
    if name == "wrap_heavy":
        return phantom.config_wrap_heavy(seed=1000)
    return phantom.acquisition(1024, 512, 181, na=1.2, seed=4000)


def build():
    """The Release-flag binaries (--use_fast_math, as the reference ships) and IEEE ones;
    returns the pipeline binaries (the Algorithm B ones, ref_qpib, sit beside them)."""
    if not os.path.isdir(os.path.join(REF, "src")):
        raise SystemExit("oracle/_ref/refcuda/src is missing: run oracle/refcuda/assemble.py <reference root> first")
    subprocess.check_call(["make", "-s", "-j4", "-C", HERE])
    subprocess.check_call(["make", "-s", "-j4", "-C", HERE, "VARIANT=ieee"])
    return {"release": os.path.join(REF, "ref_pipeline"), "ieee": os.path.join(REF, "ieee", "ref_pipeline")}


def fastuw_maps(m=256, count=4, seed=7000):
    """Wrapped phase maps of smooth surfaces (several wraps across the map) with mild noise."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:m, 0:m] / m
    maps = []
    for k in range(count):
        a, b, c = rng.uniform(4, 8), rng.uniform(1.5, 3), rng.uniform(1.5, 3)
        true = a * np.sin(b * x + k) * np.cos(c * y) + 3 * x + 0.02 * rng.standard_normal((m, m))
        maps.append(wrap(true))
    return np.stack(maps).astype(np.float32)


def fastuw_parity(O, exes, maps, ctx=None):
    """FastUnwrapping: the reference's own function (FTUP plans at the (2M)^2 its code
    transforms) and, given a context, this library's, against the FP64 oracle: the input
    normalised in place, and the unwrapped map (pixels within 1e-3 of the oracle's; the
    congruence rounding of a pixel near a half turn may differ by 2 pi)."""
    A, m = maps.shape[0], maps.shape[1]
    oracle = [O.fast_unwrap(maps[a].astype(np.float64)) for a in range(A)]

    def errors(unw, norm):
        agree = [float(np.mean(np.abs(unw[a] - oracle[a][0]) < 1e-3)) for a in range(A)]
        nerr = [float(np.sqrt(np.mean((norm[a] - oracle[a][1]) ** 2))) for a in range(A)]
        return {"agree_fraction_min": min(agree), "normalised_rmse_max": max(nerr)}

    out = {"maps": A, "side": m}
    with tempfile.TemporaryDirectory() as tmp:
        fin = os.path.join(tmp, "in.bin")
        with open(fin, "wb") as f:
            f.write(b"CTDMFU01")
            f.write(np.array([m, A], np.int32).tobytes())
            f.write(np.ascontiguousarray(maps, np.float32).tobytes())
        for kind, exe in exes.items():
            fexe = os.path.join(os.path.dirname(exe), "ref_fastuw")
            prefix = os.path.join(tmp, kind)
            r = subprocess.run([fexe, fin, prefix], capture_output=True, text=True, timeout=1800)
            if r.returncode != 0:
                raise SystemExit(f"ref_fastuw failed ({r.returncode}): {r.stderr[-2000:]}")
            info = json.loads(r.stdout.strip().splitlines()[-1])
            unw = np.fromfile(prefix + ".unwrapped.f32", np.float32).reshape(A, m, m)
            norm = np.fromfile(prefix + ".normalised.f32", np.float32).reshape(A, m, m)
            out[f"reference_{kind}"] = dict(errors(unw, norm), ms_per_map=info["ms_per_map"])
    if ctx is not None:
        import torch
        dev = torch.device("cuda", 0)
        t = torch.from_numpy(np.ascontiguousarray(maps)).to(dev)
        o = torch.zeros_like(t)
        ctx.unwrap_fast(t, o, A, m)
        torch.cuda.synchronize()
        out["this_library"] = errors(o.cpu().numpy(), t.cpu().numpy())
    return out


def residue_maps(seed=7100):
    """Wrapped phase maps with many residues: noisy tilted surfaces at three noise levels on
    256^2, a ragged 100 x 37 one (the border rules of both edges), and a map drawn from
    {0, +-pi, +-pi/2, +-1e-7} in float, whose differences land on the remainder's
    boundaries (exactly +-pi, +-2 pi, and values that round to them)."""
    rng = np.random.default_rng(seed)
    out = []
    for m, n, noise in [(256, 256, 0.6), (256, 256, 1.2), (256, 256, 2.5), (100, 37, 1.0)]:
        y, x = np.mgrid[0:n, 0:m]
        true = 0.7 * x + 0.2 * y + 3 * np.sin(x / 11.0) + noise * rng.standard_normal((n, m))
        out.append(wrap(true).astype(np.float32))
    pi = np.float32(np.pi)
    vals = np.array([0, pi, -pi, pi / 2, -pi / 2, 1e-7, -1e-7], np.float32)
    out.append(vals[rng.integers(0, len(vals), (128, 128))])
    return out


def residues_parity(O, exes, maps, ctx=None):
    """Goldstein residues: the reference's own cudaPhaseResidues (each build) and, given a
    context, this library's ctdm_goldstein charges, against the oracle's
    or_goldstein_residues, map by map: the count of differing pixels (0 is bit-exact) and
    the residue count."""
    out = {"maps": [f"{m.shape[1]}x{m.shape[0]}" for m in maps]}
    orc = [O.goldstein_residues(m) for m in maps]
    out["residues_oracle"] = [int(np.count_nonzero(q)) for q in orc]
    with tempfile.TemporaryDirectory() as tmp:
        for kind, exe in exes.items():
            rexe = os.path.join(os.path.dirname(exe), "ref_residues")
            diff, ms = [], []
            for i, m in enumerate(maps):
                fin, prefix = os.path.join(tmp, f"in{i}.bin"), os.path.join(tmp, f"{kind}{i}")
                with open(fin, "wb") as f:
                    f.write(b"CTDMRS01")
                    f.write(np.array([m.shape[1], m.shape[0], 1], np.int32).tobytes())
                    f.write(np.ascontiguousarray(m, np.float32).tobytes())
                r = subprocess.run([rexe, fin, prefix], capture_output=True, text=True, timeout=600)
                if r.returncode != 0:
                    raise SystemExit(f"ref_residues failed ({r.returncode}): {r.stderr[-2000:]}")
                ms.append(json.loads(r.stdout.strip().splitlines()[-1])["ms_per_map"])
                q = np.fromfile(prefix + ".charges.f32", np.float32).reshape(m.shape)
                diff.append(int(np.count_nonzero(q != orc[i])))
            out[f"reference_{kind}"] = {"pixels_differing": diff, "ms_per_map": ms}
    if ctx is not None:
        import torch
        dev = torch.device("cuda", 0)
        diff = []
        for i, m in enumerate(maps):
            h, w = m.shape
            q = torch.zeros((1, h, w), dtype=torch.int8, device=dev)
            c = torch.zeros((1, h, w), dtype=torch.uint8, device=dev)
            o = torch.zeros((1, h, w), dtype=torch.float32, device=dev)
            ctx.goldstein(torch.from_numpy(np.ascontiguousarray(m)).to(dev), q, c, o, 1, w, h)
            torch.cuda.synchronize()
            diff.append(int(np.count_nonzero(q[0].cpu().numpy() != orc[i])))
        out["this_library"] = {"pixels_differing": diff}
    return out


def qpib_workload(n=1024, angles=16, seed=6000):
    """Holograms with the carrier along x, as QPI Algorithm B (a 1-D filter along x) needs."""
    from ctdm_gb300 import phantom
    return phantom.acquisition(n, n // 4, angles, seed=seed, pixel=0.1e-6 * 256 / n, carrier=(0.25, 0.0))


def qpib_parity(O, exes, acq, ctx=None):
    """QPI Algorithm B: the reference's own extractQPI_AlgorithmB + calcWrapPhase (both
    builds) and, given a context, this library's ctdm_qpi_b, against the FP64 oracle on
    the same holograms: carrier column, worst-frame wrapped-phase RMS and amplitude RMS.
    The job loop's order: frame 1 takes its own carrier column, the background and every
    later frame the background's."""
    A, n = len(acq.ang_x), acq.n_holo
    m = n // 4
    ocb, ocs = O.qpib_center(acq.background), O.qpib_center(acq.holograms[0])
    bgf = O.qpib_field(acq.background, ocb)
    oracle_maps = [O.wrap_phase(O.qpib_field(acq.holograms[a], ocs if a == 0 else ocb), bgf) for a in range(A)]

    def errors(ph, am):
        pe = [float(np.sqrt(np.mean(wrap(ph[a] - oracle_maps[a][0]) ** 2))) for a in range(A)]
        ae = [float(np.sqrt(np.mean((am[a] - oracle_maps[a][1]) ** 2))) for a in range(A)]
        return {"wrapped_phase_rms_rad_max": max(pe), "amplitude_rmse_max": max(ae)}

    out = {"frames": A, "hologram": n, "carrier_column_oracle": ocb, "carrier_column_frame1_oracle": ocs}
    with tempfile.TemporaryDirectory() as tmp:
        fin = os.path.join(tmp, "in.bin")
        write_input(fin, acq, 1, (0, 0, 0))
        for kind, exe in exes.items():
            qexe = os.path.join(os.path.dirname(exe), "ref_qpib")
            prefix = os.path.join(tmp, kind)
            r = subprocess.run([qexe, fin, prefix], capture_output=True, text=True, timeout=1800)
            if r.returncode != 0:
                raise SystemExit(f"ref_qpib failed ({r.returncode}): {r.stderr[-2000:]}")
            info = json.loads(r.stdout.strip().splitlines()[-1])
            ph = np.fromfile(prefix + ".phase.f32", np.float32).reshape(A, m, m)
            am = np.fromfile(prefix + ".amp.f32", np.float32).reshape(A, m, m)
            out[f"reference_{kind}"] = dict(errors(ph, am), carrier_column=info["carrier_column"],
                                            ms_per_frame=info["ms_per_frame"],
                                            non_finite=int(np.count_nonzero(~np.isfinite(ph)) +
                                                           np.count_nonzero(~np.isfinite(am))))
    if ctx is not None:
        import torch
        dev = torch.device("cuda", ctx.device if hasattr(ctx, "device") else 0)
        ph = torch.zeros((A, m, m), dtype=torch.float32, device=dev)
        am = torch.zeros_like(ph)
        cb, cs = ctx.qpi_b(n, torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev),
                           ph, am, A)
        torch.cuda.synchronize()
        out["this_library"] = dict(errors(ph.cpu().numpy(), am.cpu().numpy()), carrier_column=cb,
                                   carrier_column_frame1=cs)
    return out


def run_reference(exe, fin, reps, R, dump=None):
    """Runs the binary; with `dump` (a folder) it also writes the reference's
    intermediate arrays there (one more, untimed repetition)."""
    with tempfile.TemporaryDirectory() as tmp:
        fout = os.path.join(tmp, "out.bin")
        cmd = [exe, fin, fout, str(reps + 1 if dump else reps)] + ([dump] if dump else [])
        r = subprocess.run(cmd, capture_output=True, text=True, timeout=3000)
        if r.returncode != 0:
            raise SystemExit(f"ref_pipeline failed ({r.returncode}): {r.stderr[-2000:]}")
        timing = json.loads(r.stdout.strip().splitlines()[-1])
        return timing, np.fromfile(fout, np.complex64).reshape(R, R, R)


def wrap(x):
    return np.angle(np.exp(1j * x))


def stage_parity(O, acq, car, dump):
    """The reference's own intermediate arrays (IEEE build) against the FP64 oracle on the
    same holograms: wrapped phase and amplitude of calcWrapPhase, the DCT unwrap, the Ewald
    hit counts and F2 of initial_F_and_F2."""
    A, m, R = len(acq.ang_x), acq.m_crop, acq.r_vol
    ph = np.fromfile(os.path.join(dump, "phase.f32"), np.float32).reshape(A, m, m)
    am = np.fromfile(os.path.join(dump, "amp.f32"), np.float32).reshape(A, m, m)
    uw = np.fromfile(os.path.join(dump, "unwrapped.f32"), np.float32).reshape(A, m, m)
    bgf = O.qpi_field(acq.background, m, *car)
    ph_err, am_err, uw_err = [], [], []
    for a in range(A):
        oph, oam = O.wrap_phase(O.qpi_field(acq.holograms[a], m, *car), bgf)
        ph_err.append(float(np.sqrt(np.mean(wrap(ph[a] - oph) ** 2))))
        am_err.append(float(np.sqrt(np.mean((am[a] - oam) ** 2))))
        ouw = O.dct_unwrap(oph, 0)
        uw_err.append(float(np.sqrt(np.mean((uw[a] - ouw) ** 2))))
    del ph, am, uw
    par = O.make_params(acq.n_holo, m, R, 0, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med, carrier=car)
    oph, oam, _ = O.front_end(par, acq.holograms, acq.background)
    U = np.stack([O.rytov_spectrum(oph[a], oam[a]) for a in range(A)])
    del oph, oam
    oF2, oC = O.ewald_map(U, acq.ang_x, acq.ang_y, acq.fm0, acq.df, acq.dx)
    del U
    rc = np.fromfile(os.path.join(dump, "counts.f32"), np.float32).reshape(R, R, R)
    rf2 = np.fromfile(os.path.join(dump, "f2.c64"), np.complex64).reshape(R, R, R)
    same = rc.astype(np.int64) == oC.astype(np.int64)
    both = same & (oC > 0)
    d = rf2[both].astype(np.complex128) - oF2[both]
    f2_rel = float(np.linalg.norm(d) / np.linalg.norm(oF2[both]))
    return {"wrapped_phase_rms_rad_max": max(ph_err), "wrapped_phase_rms_rad_mean": float(np.mean(ph_err)),
            "amplitude_rmse_max": max(am_err), "dct_unwrapped_rmse_rad_max": max(uw_err),
            "hit_count_voxels_equal_fraction": float(np.mean(same)),
            "hit_voxels_reference": int(np.count_nonzero(rc)), "hit_voxels_oracle": int(np.count_nonzero(oC)),
            "hit_voxels_differing": int(np.count_nonzero(~same)),
            "f2_rel_l2_on_equal_hit_voxels": f2_rel}


def finite_rmse(a, ref):
    """RMSE over the voxels where `a` is finite, and the count of the others."""
    ok = np.isfinite(a.real) & np.isfinite(a.imag)
    bad = int(ok.size - np.count_nonzero(ok))
    if not ok.any():
        return None, bad
    d = a[ok].astype(np.complex128) - ref[ok]
    return float(np.sqrt(np.mean(np.abs(d) ** 2))), bad


def write_input(path, acq, iters, carrier):
    with open(path, "wb") as f:
        f.write(b"CTDMREF1")
        f.write(np.array([acq.n_holo, acq.r_vol, len(acq.ang_x), iters, *carrier], np.int32).tobytes())
        f.write(np.array([acq.n_med, acq.wavelength, acq.dx], np.float64).tobytes())
        f.write(np.ascontiguousarray(acq.ang_x, np.float32).tobytes())
        f.write(np.ascontiguousarray(acq.ang_y, np.float32).tobytes())
        f.write(np.ascontiguousarray(acq.background, np.float32).tobytes())
        f.write(np.ascontiguousarray(acq.holograms, np.float32).tobytes())


def rmse(a, b):
    return float(np.sqrt(np.mean(np.abs(a.astype(np.complex128) - b.astype(np.complex128)) ** 2)))


def ours(acq, iters, goldstein, reps):
    import torch
    import ctdm_gb300 as C
    ctx = C.Context(0)
    dev = torch.device("cuda", 0)
    r = acq.r_vol
    out = {}
    for gold in sorted({False, goldstein}):
        p = C.params_for(acq, iters, run_goldstein=int(gold))
        h16, b16 = acq.holograms.astype(np.uint16), acq.background.astype(np.uint16)
        # one pageable output volume for every call, as the reference's harness keeps its own
        vol = np.empty((r, r, r), np.complex64)
        ctx.reconstruct(p, h16, b16, acq.ang_x, acq.ang_y, out=vol)          # warm (autotune, buffers)
        torch.cuda.synchronize()
        t = []
        for _ in range(reps):
            t0 = time.perf_counter()
            ctx.reconstruct(p, h16, b16, acq.ang_x, acq.ang_y, out=vol)
            t.append((time.perf_counter() - t0) * 1e3)
        holo, bg = torch.from_numpy(acq.holograms).to(dev), torch.from_numpy(acq.background).to(dev)
        d = torch.empty((r, r, r), dtype=torch.complex64, device=dev)
        ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, d)
        torch.cuda.synchronize()
        td = []
        for _ in range(reps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            ctx.reconstruct_device(p, holo, bg, acq.ang_x, acq.ang_y, d)
            b.record()
            b.synchronize()
            td.append(a.elapsed_time(b))
        out["goldstein" if gold else "plain"] = {"host_buffers_ms_mean": float(np.mean(t)),
                                                 "device_resident_ms_mean": float(np.mean(td)), "volume": vol}
        del holo, bg, d
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--configs", default="plain_small,wrap_heavy,plain_512")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=None)
    ap.add_argument("--qpib", action="store_true",
                    help="only QPI Algorithm B: the reference's own against the oracle and this library")
    ap.add_argument("--fastuw", action="store_true",
                    help="only FastUnwrapping: the reference's own against the oracle and this library")
    ap.add_argument("--residues", action="store_true",
                    help="only the Goldstein residues: the reference's own against the oracle and this library")
    args = ap.parse_args()
    import oracle as O
    from ctdm_gb300 import build as cbuild
    cbuild.build()
    exes = build()
    if args.qpib or args.fastuw or args.residues:
        import ctdm_gb300 as C
        line = (qpib_parity(O, exes, qpib_workload(), C.Context(0)) if args.qpib
                else fastuw_parity(O, exes, fastuw_maps(), C.Context(0)) if args.fastuw
                else residues_parity(O, exes, residue_maps(), C.Context(0)))
        print(json.dumps(line))
        if args.out:
            with open(args.out, "w") as f:
                json.dump(line, f, indent=1)
        return
    lines = []
    for name in args.configs.split(","):
        iters, gold = CONFIGS[name]
        acq = workload(name)
        car = O.qpi_carrier(acq.background)
        R = acq.r_vol
        refs = {}
        with tempfile.TemporaryDirectory() as tmp:
            fin = os.path.join(tmp, "in.bin")
            write_input(fin, acq, iters, car)
            dump = os.path.join(tmp, "dump")
            os.makedirs(dump)
            for kind, exe in exes.items():
                refs[kind] = run_reference(exe, fin, args.reps, R, dump=dump if kind == "ieee" else None)
            stages = stage_parity(O, acq, car, dump)
        par = O.make_params(acq.n_holo, acq.m_crop, R, iters, acq.fm0, acq.df, acq.dx, acq.k2, acq.n_med)
        fp64, ocar, _ = O.tomogram(par, acq.holograms, acq.background, acq.ang_x, acq.ang_y)
        mine = ours(acq, iters, gold, args.reps)
        plain = mine["plain"]
        ref_out = {}
        for kind, (timing, vol) in refs.items():
            err, bad = finite_rmse(vol, fp64)
            ref_out[kind] = {"ms_per_tomogram": timing["ms_mean"], "ms_best": timing["ms_best"],
                             "front_end_ms": timing["front_ms_mean"], "batchrecon_ms": timing["recon_ms_mean"],
                             "ri_rmse_vs_fp64_finite_voxels": err, "non_finite_voxels": bad,
                             "non_finite_map_values": timing.get("non_finite_map_values"),
                             "build": ("nvcc --use_fast_math (the reference's Release flags)" if kind == "release"
                                       else "nvcc without fast math") + ", cuFFT",
                             "span": "host holograms -> RI volume on the host"}
        ieee_vol = refs["ieee"][1]
        line = {
            "workload": name, "holograms": f"{len(acq.ang_x)}x{acq.n_holo}^2", "volume": f"{R}^3",
            "iterations": iters, "carrier": list(car), "reference_cuda": ref_out,
            "this_library": {k: {"host_buffers_ms": v["host_buffers_ms_mean"],
                                 "device_resident_ms": v["device_resident_ms_mean"],
                                 "ri_rmse_vs_fp64": rmse(v["volume"], fp64),
                                 "ri_rmse_vs_reference_cuda_ieee": finite_rmse(v["volume"], ieee_vol.astype(np.complex128))[0]
                                 if np.isfinite(ieee_vol).all() else None} for k, v in mine.items()},
            "reference_stages_vs_fp64": stages,
            "speedup_host_buffers_same_work": refs["release"][0]["ms_mean"] / plain["host_buffers_ms_mean"],
            "reps": args.reps,
        }
        print(json.dumps(line))
        lines.append(line)
    if args.out:
        with open(args.out, "w") as f:
            json.dump(lines, f, indent=1)


if __name__ == "__main__":
    main()
