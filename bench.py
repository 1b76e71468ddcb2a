"""Benchmark of the GB300 halo painter on the reference's headline workload.

Workload (one "step"): a synthetic catalogue of 1e7 halos (10 float32 per record, shell
100-8000 Mpc, masses 1e12-3e15 Msun/h, seed 2) painted to two HEALPix Nside 4096 maps,
tSZ Compton-y (nu = 0 table, profile 1) and kSZ (profile 2), zmax = 6, model 1:
radial/mass cut, per-halo set-up, disc enumeration, profile interpolation, deposit, and
the float32 read-out of both maps.  Inputs (400 MB) and maps (2 x 805 MB) exceed L2, so
no explicit flush is needed between steps.

  value  halos/s with the catalogue resident in HBM (CUDA events on the paint stream)
  e2e    halos/s through the C ABI with host buffers: pinned catalogue H2D, paint, and
         both float maps copied back to pinned host memory, every step

--impl reference times the CPU implementation of the path on the host cores instead:
the oracle (a C restatement of pks2map, threads as MPI ranks with private float maps and
a final sum) over the same whole catalogue every step, generated and painted without
loading the GPU library.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_HALOS = 10_000_000
NSIDE = 4096
SHELL = (100.0, 8000.0)
MASS = (1e12, 3e15)
SEED = 2
ZMAX = 6.0
MAPS = ((0, 1), (0, 2))
LAUNCHES_PER_STEP = 15
# DRAM bytes (read + write) per pixel update of k_paint_halos from an ncu capture of this
# workload's launch (1e7 halos at Nside 4096, one pass: dram__bytes_read.sum +
# dram__bytes_write.sum = 1.20 GB + 0.61 GB for 3.51e7 updates on each of two maps)
PAINT_DRAM_BYTES_PER_UPDATE = 51.6
# L2 atomic throughput of this GB300 (sectors/s): ncu lts__t_sectors_srcunit_tex_op_atom
# of the same capture, 26.7 sectors/ns at 7.06 % of peak sustained
L2_ATOMIC_SECTORS_PER_S = 3.79e11
METRIC = "halos/sec & pixel-updates/sec at Nside=4096, 1 GB300; rel err vs FP64 oracle"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--halos", type=int, default=N_HALOS)
    ap.add_argument("--nside", type=int, default=NSIDE)
    ap.add_argument("--no-plain", action="store_true", help="skip the FP64 drop-in comparison")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-files", action="store_true",
                    help="skip the command line's end-to-end run (file read to FITS written)")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the check of this run's maps and pixel sets against the oracle")
    ap.add_argument("--cl-lmax", type=int, default=2047,
                    help="lmax of the C_l ratio of the Nside 4096 maps (0: skip)")
    ap.add_argument("--no-precision-form", action="store_true",
                    help="skip the precision-form report (1e5 halos, Nside 512 + 8192^2 flat sky)")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the default launch parameters instead of p2m_autotune's choice")
    ap.add_argument("--no-multi-table", action="store_true",
                    help="skip the multi-table form (5e7 halos in 4M chunks, six Nside 4096 maps)")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the ensemble form (64 light-cones, one Nside 1024 map each)")
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def wait_first(self, timeout=5.0):
        """Block until nvidia-smi has produced its first sample (it takes a moment to
        start), so that the samples cover the timed region that follows."""
        t0 = time.time()
        while self.proc is not None and not self.lines and time.time() - t0 < timeout:
            time.sleep(0.01)

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[1:]:  # the first sample precedes the timed region
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(x, device=None):
    """The largest of x over the ranks of the default process group (x itself without
    one): every replica's time enters the whole-job throughput through the slowest."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(units_per_rank, world_size, ms_max):
    """Whole-job units/s of replicas that each process units_per_rank, timed by the
    slowest rank (weak scaling: the work per replica is fixed)."""
    return units_per_rank * world_size / (ms_max * 1e-3)


def map_errors(a, b):
    """Error of map a against the FP64 map b: per-pixel max-abs, relative L2, the largest
    relative error where |b| > 1e-3 max|b|, and the total's error relative to the total
    and to sum|b| (the two differ for the signed kSZ map)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    mx = np.abs(b).max()
    mask = np.abs(b) > 1e-3 * mx
    rel = np.abs(a[mask] - b[mask]) / np.abs(b[mask])
    return {"max_rel_masked": float(rel.max()) if rel.size else 0.0,
            "max_abs": float(np.abs(a - b).max()),
            "rel_l2": float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)),
            "total_rel": float(abs(a.sum() - b.sum()) / max(abs(b.sum()), 1e-300)),
            "total_rel_abs": float(abs(a.sum() - b.sum()) / max(np.abs(b).sum(), 1e-300))}


def cl_ratio(spec, lmin=1):
    """max and rms of |C(a) / C(b) - 1| over the multipoles (or bins) from lmin on where
    C(b) is nonzero, from a spectra dict with "aa" (map a) and "bb" (the FP64 map b)."""
    aa, bb = np.asarray(spec["aa"])[lmin:], np.asarray(spec["bb"])[lmin:]
    sel = bb > 0
    d = np.abs(aa[sel] / bb[sel] - 1.0)
    return {"max": float(d.max()) if d.size else None,
            "rms": float(np.sqrt(np.mean(d * d))) if d.size else None}


def precision_form(device):
    """The precision form of the path: the 1e5-halo catalogue (seed 1, shell 100-3000 Mpc,
    masses 1e12-1e15) painted with the 148 GHz alpha = 0 table to a HEALPix Nside 512 tSZ
    map and a flat-sky 8192^2 map over 10 degrees, by the mixed painter (FP32 profile
    values, compensated FP32 accumulation) and by the FP64-accumulating painter.  Reports
    the per-map errors of the mixed maps against the FP64 maps, the C_l ratio (l <= 1535 on
    the sphere, 100 bins of ell <= 8000 on the flat sky) and the paint times."""
    import torch

    import matt_young_mapmaking_gb300 as p2m
    n, nside, nfs, fov = 100_000, 512, 8192, 10.0
    rec = p2m.generate_catalogue(1, n, 10, r=(100.0, 3000.0), m=(1e12, 1e15))
    d_rec = torch.from_numpy(rec).to(torch.device("cuda", device))
    table = p2m.make_maptable(1, 148.0, 0.0, device=device)
    maps, times = {}, {}
    for prec in ("mixed", "fp64"):
        with p2m.Painter(nside=nside, npix_fs=nfs, fov_deg=fov, precision=prec,
                         maps=((0, 1),), max_records=n, device=device) as pt:
            pt.load_table(0, table)
            ts = []
            for _ in range(6):
                pt.reset()
                torch.cuda.synchronize(device)
                t0 = time.perf_counter()
                pt.paint_records_device(d_rec.data_ptr(), n, 10)
                pt.flush()
                pt.synchronize()
                ts.append(time.perf_counter() - t0)
            times[prec] = 1e3 * float(np.median(ts[1:]))
            maps[prec] = (pt.healpix(0), pt.flatsky(0))
    hp_cl = p2m.cl_healpix(maps["mixed"][0], maps["fp64"][0], lmax=3 * nside - 1,
                           device=device)
    fs_cl = p2m.cl_flatsky(maps["mixed"][1], maps["fp64"][1], fov_rad=np.radians(fov),
                           ell_max=8000.0, nbins=100, device=device)
    return {"workload": "%d halos (seed 1, 100-3000 Mpc, 1e12-1e15), 148 GHz table, "
                        "HEALPix Nside %d + flat sky %d^2 over %g deg" % (n, nside, nfs, fov),
            "ms_mixed": times["mixed"], "ms_fp64": times["fp64"],
            "halos_per_s_mixed": n / (times["mixed"] * 1e-3),
            "timing": "wall clock around paint + read-out, median of 5 after one warm-up",
            "healpix": dict(map_errors(maps["mixed"][0], maps["fp64"][0]),
                            cl_ratio=dict(cl_ratio(hp_cl), lmax=3 * nside - 1)),
            "flatsky": dict(map_errors(maps["mixed"][1], maps["fp64"][1]),
                            cl_ratio=dict(cl_ratio(fs_cl, lmin=0), ell_max=8000.0, bins=100))}


def multi_table_form(device, steps=3, warmup=1):
    """The multi-table form: 5e7 halos (seed 4, shell 100-8000 Mpc, masses 1e12-3e15)
    streamed from pinned host memory in 4M-halo paint calls (each streamed in 2M-record
    chunks that overlap their copies with the cut) into six Nside 4096 maps in one
    enumeration: tSZ at 148, 200, 218, 353 and 545 GHz, each from its own table, and kSZ.
    Timed with CUDA events from the first copy to the six maps ready on the device; the
    read-out of the six maps to pinned host memory is timed beside it.  The mixed maps
    are compared with the FP64-accumulating painter's."""
    import torch

    import matt_young_mapmaking_gb300 as p2m
    n, chunk, nside = 50_000_000, 4_000_000, 4096
    freqs = (148.0, 200.0, 218.0, 353.0, 545.0)
    maps = tuple((t, 1) for t in range(len(freqs))) + ((0, 2),)
    h_rec = torch.empty((n, 10), dtype=torch.float32).pin_memory()
    for a in range(0, n, 10_000_000):
        m = min(10_000_000, n - a)
        h_rec[a:a + m] = torch.from_numpy(
            p2m.generate_catalogue(4, m, 10, r=SHELL, m=MASS, first=a))
    rec = h_rec.numpy()
    tables = [p2m.make_maptable(1, f, 0.0, device=device) for f in freqs]
    npix = 12 * nside * nside
    h_map = torch.empty(npix, dtype=torch.float32).pin_memory()
    dev = torch.device("cuda", device)
    d_chunk = h_rec[:chunk].to(dev)
    res, got, tun = {}, {}, {}
    for prec in ("mixed", "fp64"):
        with p2m.Painter(nside=nside, precision=prec, maps=maps, zmax=ZMAX, max_records=chunk,
                         device=device) as pt:
            for t, tab in enumerate(tables):
                pt.load_table(t, tab)
            # set-up, outside the timed region: launch parameters chosen by the library's
            # autotuner on one chunk of this catalogue
            tun[prec] = pt.autotune(d_chunk.data_ptr(), chunk, 10, reps=2)

            def step():
                pt.reset()
                for a in range(0, n, chunk):
                    pt.paint_records(rec[a:a + chunk])
                pt.flush()

            for _ in range(warmup):
                step()
            torch.cuda.synchronize(dev)
            t0 = time.perf_counter()
            for _ in range(steps):
                step()
                pt.synchronize()
            ms = 1e3 * (time.perf_counter() - t0) / steps
            t0 = time.perf_counter()
            for m in range(len(maps)):
                pt.healpix_into(m, h_map.data_ptr())
            rd_ms = 1e3 * (time.perf_counter() - t0)
            st = pt.stats()
            res[prec] = {"ms_per_step": ms, "halos_per_s": n / (ms * 1e-3),
                         "pixel_updates_per_s": st["hp_updates"] * len(maps) / (ms * 1e-3),
                         "readout_ms": rd_ms, "tuning": tun[prec]}
            got[prec] = [pt.healpix(m) for m in range(len(maps))]
    names = ["tsz_%dghz" % f for f in freqs] + ["ksz"]
    errs = {nm: map_errors(got["mixed"][m], got["fp64"][m]) for m, nm in enumerate(names)}
    return {"workload": "%d halos in %d-halo paint calls from pinned host memory, six HEALPix "
                        "Nside %d maps (tSZ 148/200/218/353/545 GHz, each from its own table, "
                        "+ kSZ), zmax %g" % (n, chunk, nside, ZMAX),
            "timing": "wall clock around %d steps of reset + streamed paint + sweep, "
                      "synchronised per step; readout_ms: the six maps to pinned host memory"
                      % steps,
            "mixed": res["mixed"], "fp64": res["fp64"],
            "speedup_of_mixed": res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"],
            "error_vs_fp64": errs}


def ensemble_form(device, steps=20, warmup=3):
    """The ensemble form: 64 independent light-cones of uneven size (halo counts
    log-uniform in 1e4-1e6 and shell depths log-uniform in 1000-6000 Mpc, both drawn with
    seed 5; cone i's catalogue from seed 5000 + i, masses 1e12-3e15), each painted to its
    own Nside 1024 tSZ y map (nu = 0 table) in one call: the per-cone offset table goes in
    with the concatenated records, and one enumeration and one painting launch serve all
    cones.  Aggregate halos/s with the records resident (CUDA events around reset, paint
    and read-out of all 64 maps), and per-cone errors of the compensated FP32 maps against
    the FP64-accumulating painter."""
    import torch

    import matt_young_mapmaking_gb300 as p2m
    ncones, nside = 64, 1024
    rng = np.random.default_rng(5)
    counts = np.exp(rng.uniform(np.log(1e4), np.log(1e6), ncones)).astype(np.int64)
    depths = np.exp(rng.uniform(np.log(1000.0), np.log(6000.0), ncones))
    recs = [p2m.generate_catalogue(5000 + i, int(counts[i]), 10, r=(100.0, float(depths[i])),
                                   m=(1e12, 3e15)) for i in range(ncones)]
    off = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    dev = torch.device("cuda", device)
    d_rec = torch.from_numpy(np.concatenate(recs)).to(dev)
    n = int(off[-1])
    del recs
    table = p2m.make_maptable(1, 0.0, 0.0, device=device)
    stream = torch.cuda.Stream(device=dev)
    res, maps = {}, {}
    for prec in ("mixed", "fp64"):
        with p2m.Painter(nside=nside, precision=prec, maps=((0, 1),), zmax=6.0, max_records=n,
                         device=device, ncones=ncones) as pt:
            pt.load_table(0, table)

            def step():
                pt.reset()
                pt.paint_ensemble_device(d_rec.data_ptr(), off, 10, stream.cuda_stream)
                pt.flush()

            for _ in range(warmup):
                step()
            torch.cuda.synchronize(dev)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record(stream)
            for _ in range(steps):
                step()
            pt.synchronize()
            ev1.record(stream)
            torch.cuda.synchronize(dev)
            ms = ev0.elapsed_time(ev1) / steps
            st = pt.stats()
            res[prec] = {"ms_per_step": ms, "halos_per_s": n / (ms * 1e-3),
                         "pixel_updates_per_s": st["hp_updates"] / (ms * 1e-3)}
            maps[prec] = pt.healpix(0).reshape(ncones, -1)
    errs = [map_errors(maps["mixed"][c], maps["fp64"][c]) for c in range(ncones)
            if np.any(maps["fp64"][c])]
    return {"workload": "%d light-cones, %d halos in all (%d-%d per cone), shells 100 Mpc to "
                        "%d-%d Mpc, one HEALPix Nside %d tSZ y map each"
                        % (ncones, n, counts.min(), counts.max(), depths.min(), depths.max(), nside),
            "mixed": res["mixed"], "fp64": res["fp64"],
            "speedup_of_mixed": res["fp64"]["ms_per_step"] / res["mixed"]["ms_per_step"],
            "timing": "CUDA events around %d steps of reset + paint + read-out of all maps, "
                      "records resident" % steps,
            "per_cone_error": {k: float(max(e[k] for e in errs)) for k in
                               ("max_rel_masked", "rel_l2", "total_rel")},
            "per_cone_error_note": "largest over the cones of each cone's error"}


def workload_name(n, nside):
    """config.workload of both arms (the same string for the same workload)"""
    return ("pks2map c2: %d halos x 10 float, shell %g-%g Mpc, masses %g-%g, HEALPix Nside %d, "
            "tSZ y + kSZ, zmax %g" % (n, SHELL[0], SHELL[1], MASS[0], MASS[1], nside, ZMAX))


def catalogue(n):
    import matt_young_mapmaking_gb300 as p2m
    return p2m.generate_catalogue(SEED, n, 10, r=SHELL, m=MASS)


def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    return oracle


def oracle_catalogue(n):
    """The same catalogue, generated by the oracle's restatement of the generator (the
    CPU arm loads no library of the product)"""
    return _oracle().generate_catalogue(SEED, n, 10, r=SHELL, m=MASS)


def oracle_table():
    """Full-size make_maptable table (model 1, nu = 0) from the oracle, cached in /tmp."""
    oracle = _oracle()
    path = "/tmp/p2m_table_model1_nu0_full.bin"
    if os.path.exists(path) and os.path.getsize(path) == 36 + 8 * 100 * 100 * 200:
        with open(path, "rb") as f:
            return f.read()
    img = oracle.make_maptable(1, 0.0, 0.0)
    with open(path + ".tmp", "wb") as f:
        f.write(img)
    os.replace(path + ".tmp", path)
    return img


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), and its core count"""
    name = None
    try:
        out = subprocess.run(["lscpu"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL,
                             text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    if not name:
        try:
            with open("/proc/cpuinfo") as f:
                info = f.read()
            for key in ("model name", "Model", "CPU part"):
                for line in info.splitlines():
                    if line.startswith(key):
                        name = line.split(":", 1)[1].strip()
                        break
                if name:
                    break
        except Exception:
            pass
    return "%s, %d cores" % (name or "unknown", os.cpu_count() or 1)


def cpu_reference(rec, nside, threads, table, steps, warmup):
    """The reference's CPU implementation of the path, timed on the host cores: the
    oracle's halo loop in the reference's FP32 mode with `threads` threads standing in for
    its MPI ranks.  Every step is one whole pks2map run over the whole catalogue: each
    rank zeroes its private float maps (hpmapl = 0, pks2map.f90:278-279), paints its
    contiguous block of records (pksc.f90:51-52), and the ranks' maps are summed in rank
    order (MPI_Allreduce, pks2map.f90:313-314).  Returns the step times (s) and a
    description."""
    oracle = _oracle()
    tab = oracle.Table(table)
    p = oracle.params(nside=nside, npix_fs=0, maps=MAPS, zmax=ZMAX, fp32=True, nfloat=10)
    t0 = time.perf_counter()
    rm = oracle.RankMaps(p, threads)
    t_alloc = time.perf_counter() - t0
    times, st = [], None
    for i in range(warmup + steps):
        t0 = time.perf_counter()
        rm.zero()
        st = rm.paint(p, [tab], rec)
        rm.reduce(threads)
        if i >= warmup:
            times.append(time.perf_counter() - t0)
    del rm
    t_med = float(np.median(times))
    info = {"unit": "halos/s", "cores": threads, "kind": "port", "cpu": cpu_model(),
            "sample": "the whole %d-record catalogue every step: %d threads as MPI ranks, each "
                      "zeroing its private float maps (Nside %d, 2 maps), painting its block "
                      "of records, then the rank-order sum of the maps; median of %d steps "
                      "after %d warm-up (maps allocated once, %.2fs)"
                      % (len(rec), threads, nside, steps, warmup, t_alloc),
            "pixel_updates_per_s": len(MAPS) * st["hp_updates"] / t_med if t_med > 0 else None}
    return times, info


def parity_vs_oracle(rec, table, nside, maps_mixed, maps_fp64, device):
    """The GPU maps of the timed run (mixed and plain FP64 paths) and the per-record pixel
    sets of one more paint of the same catalogue, checked against the oracle's FP64 halo
    loop on the same records and table image (all host cores, orc_paint_parallel)."""
    import torch

    import matt_young_mapmaking_gb300 as p2m
    oracle = _oracle()
    t0 = time.perf_counter()
    p = oracle.params(nside=nside, maps=MAPS, zmax=ZMAX, nfloat=10)
    rhp, _, rst, rsets = oracle.paint(p, [oracle.Table(table)], rec, record_sets=True,
                                      set_cap=1 << 26, threads=os.cpu_count() or 1)
    t_oracle = time.perf_counter() - t0
    dev = torch.device("cuda", device)

    def keys(srec, spix):
        r = torch.from_numpy(np.ascontiguousarray(srec)).to(dev)
        q = torch.from_numpy(np.ascontiguousarray(spix)).to(dev)
        return torch.sort(r * (1 << 28) + q).values

    rkeys = keys(*rsets)
    del rsets
    os.environ["P2M_SET_CAP"] = str(1 << 26)
    try:
        with p2m.Painter(nside=nside, precision="mixed", maps=MAPS, zmax=ZMAX,
                         flags=p2m.FLAG_RECORD_SETS | p2m.FLAG_ALL_HALOS,
                         max_records=len(rec), device=device) as pt:
            pt.load_table(0, table)
            pt.paint_records(rec)
            gst = pt.stats()
            gkeys = keys(*pt.pixel_sets())
    finally:
        del os.environ["P2M_SET_CAP"]
    if gkeys.shape == rkeys.shape:
        mism = int((gkeys != rkeys).sum())
    else:
        mism = abs(int(gkeys.numel()) - int(rkeys.numel()))
    out = {"oracle": "FP64 halo loop of the oracle (orc_paint_parallel, %d threads, %.1fs), "
                     "same records and table image" % (os.cpu_count() or 1, t_oracle),
           "pairs_oracle": int(rkeys.numel()), "pairs_gpu": int(gkeys.numel()),
           "set_mismatches": mism,
           "hp_updates_equal": gst["hp_updates"] == rst["hp_updates"]}
    for name, got in (("mixed", maps_mixed), ("fp64", maps_fp64)):
        if got is None:
            continue
        out[name] = {nm: map_errors(got[m], rhp[m]) for m, nm in enumerate(("tsz", "ksz"))}
    return out


def e2e_files(rec, table, nside, precision):
    """The drop-in end to end: the pks2map command line on the headline catalogue, from the
    .pksc file read to <out>_hp.fits written (tSZ, profile 1, as one reference run paints
    one profile; flat sky at the reference's default 16^2).  Its own clock (P2M_TIMING):
    file read + paint, statistics, writes; and the whole process's wall time, CUDA
    start-up included.  Files in a temporary directory, removed afterwards."""
    import shutil
    import tempfile

    import matt_young_mapmaking_gb300 as p2m
    exe = os.path.join(ROOT, "matt_young_mapmaking_gb300", "pks2map")
    d = tempfile.mkdtemp(prefix="p2m_e2e_")
    try:
        cat, tab, out = os.path.join(d, "c2.pksc"), os.path.join(d, "table.bin"), os.path.join(d, "c2")
        p2m.write_pksc(cat, rec)
        p2m.write_table(tab, table)
        args = [exe, cat, out, tab, "0.0", str(nside), "0", "0", "16", "10.0", str(ZMAX), "0.0",
                "1", "1"]
        env = dict(os.environ, P2M_TIMING="1", P2M_PRECISION=precision)
        runs = []
        for _ in range(3):
            t0 = time.perf_counter()
            r = subprocess.run(args, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True,
                               env=env, timeout=600)
            wall = time.perf_counter() - t0
            if r.returncode != 0:
                return {"error": r.stderr.strip()[-300:]}
            line = [x for x in r.stderr.splitlines() if x.startswith("pks2map timing:")][-1]
            nums = [float(x) for x in line.replace(",", " ").split() if x[0].isdigit()]
            runs.append((nums[3], nums[0], nums[1], nums[2], wall, nums[4], nums[5]))
        best = min(runs)
        size = os.path.getsize(out + "_hp.fits")
        return {"e2e_files_ms": 1e3 * best[0],
                "read_paint_ms": 1e3 * best[1], "statistics_ms": 1e3 * best[2],
                "writes_ms": 1e3 * best[3], "process_wall_ms": 1e3 * best[4],
                "of_which_setup_ms": 1e3 * best[5], "of_which_release_ms": 1e3 * best[6],
                "halos_per_s": len(rec) / best[0], "fits_bytes": size,
                "pksc_bytes": os.path.getsize(cat),
                "what": "pks2map %s <out> <table> 0.0 %d 0 0 16 10.0 %g 0.0 1 1: file read "
                        "through _hp.fits written (its own clock, best of 3 runs); "
                        "process_wall_ms adds process and CUDA start-up" % (
                            os.path.basename(cat), nside, ZMAX)}
    finally:
        shutil.rmtree(d, ignore_errors=True)


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    rec = oracle_catalogue(args.halos)
    threads = os.cpu_count() or 1
    times, info = cpu_reference(rec, args.nside, threads, oracle_table(), args.steps,
                                args.warmup)
    t = float(np.median(times))
    v = args.halos / t
    out = {"metric": METRIC, "value": v, "unit": "halos/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (Philox catalogue, seed %d)" % SEED, "impl": "reference",
           "config": {"workload": workload_name(args.halos, args.nside)},
           "timing": "wall clock of each step, median over the steps; total of the timed "
                     "steps %.2fs" % float(np.sum(times)),
           "step_times_s": [round(float(t), 4) for t in times],
           "cpu_baseline": dict(info, value=v),
           "e2e": {"value": v, "unit": "halos/s", "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    out["cpu_baseline"].pop("pixel_updates_per_s", None)
    print(json.dumps(out))


def run_ours(args):
    import torch

    import matt_young_mapmaking_gb300 as p2m
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    N, nside = args.halos, args.nside
    npix = 12 * nside * nside
    rec = catalogue(N)
    h_rec = torch.from_numpy(rec).pin_memory()
    d_rec = h_rec.to(dev)
    table = p2m.make_maptable(1, 0.0, 0.0, device=local)
    outs = [torch.empty(npix, dtype=torch.float32, device=dev) for _ in MAPS]
    h_outs = [torch.empty(npix, dtype=torch.float32).pin_memory() for _ in MAPS]
    stream = torch.cuda.Stream(device=dev)

    tunings = {}

    def make(precision):
        pt = p2m.Painter(nside=nside, precision=precision, maps=MAPS, zmax=ZMAX,
                         max_records=N, device=local, flags=p2m.FLAG_TIMING)
        pt.load_table(0, table)
        if not args.no_autotune:
            # set-up, outside the timed region: the launch parameters are chosen on this
            # catalogue by the library's autotuner
            tunings[precision] = pt.autotune(d_rec.data_ptr(), N, 10, reps=3)
        else:
            tunings[precision] = pt.tuning()
        return pt

    def step(pt):
        pt.reset()
        for m in range(len(MAPS)):  # the sweep writes the maps in place
            pt.bind_healpix_device(m, outs[m].data_ptr())
        pt.paint_records_device(d_rec.data_ptr(), N, 10, stream.cuda_stream)
        for m in range(len(MAPS)):
            pt.healpix_device(m, outs[m].data_ptr(), stream.cuda_stream)

    def barrier():
        torch.cuda.synchronize(dev)
        if ws > 1:
            torch.distributed.barrier()

    def timed(pt, steps, warmup, sampler=None):
        for _ in range(warmup):
            step(pt)
        barrier()
        if sampler:
            sampler.start()
            sampler.wait_first()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            step(pt)
        ev1.record(stream)
        barrier()
        clocks = sampler.stop() if sampler else None
        ms = max_over_ranks(ev0.elapsed_time(ev1) / steps, dev)
        return ms, clocks

    pt = make(args.precision)
    sampler = ClockSampler(local)
    ms, clocks = timed(pt, args.steps, args.warmup, sampler)
    phases = pt.timings()
    st = pt.stats()
    maps_main = [o.cpu().numpy() for o in outs]

    # end to end through the C ABI with host buffers
    def e2e_step():
        pt.reset()
        for m in range(len(MAPS)):
            pt.bind_healpix_device(m, 0)
        pt.paint_records(h_rec.numpy())
        for m in range(len(MAPS)):
            pt.healpix_into(m, h_outs[m].data_ptr())
    for _ in range(2):
        e2e_step()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    barrier()
    e2e_seq_ms = max_over_ranks(1e3 * (time.perf_counter() - t0) / args.steps, dev)

    # the same steps pipelined through the asynchronous read-out: step k's maps are
    # copied to the host while step k + 1's catalogue is copied in and painted into the
    # other of two bound buffer sets; every step still moves its catalogue in and its maps
    # out inside the timed region, and the run ends when the last maps have arrived
    d_sets = [outs, [torch.empty(npix, dtype=torch.float32, device=dev) for _ in MAPS]]
    h_sets = [h_outs, [torch.empty(npix, dtype=torch.float32).pin_memory() for _ in MAPS]]

    def e2e_pipelined_step(k):
        b = k & 1
        pt.reset()
        for m in range(len(MAPS)):
            pt.bind_healpix_device(m, d_sets[b][m].data_ptr())
        pt.paint_records(h_rec.numpy())
        for m in range(len(MAPS)):
            pt.healpix_async(m, h_sets[b][m].data_ptr())

    for k in range(2):
        e2e_pipelined_step(k)
    pt.synchronize()
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        e2e_pipelined_step(k)
    pt.synchronize()
    barrier()
    e2e_ms = max_over_ranks(1e3 * (time.perf_counter() - t0) / args.steps, dev)
    pt.close()
    # the last pipelined step's maps, as they arrived in host memory, against the resident
    # steps' maps (the same catalogue; the compensated sums agree to float rounding)
    last = h_sets[(args.steps - 1) & 1]
    e2e_check = max(map_errors(last[m].numpy(), maps_main[m])["max_rel_masked"]
                    for m in range(len(MAPS)))
    # the host link alone: the same copies without the painting
    d_tmp = torch.empty_like(h_rec, device=dev)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        d_tmp.copy_(h_rec, non_blocking=True)
    barrier()
    h2d_ms = 1e3 * (time.perf_counter() - t0) / args.steps
    t0 = time.perf_counter()
    for _ in range(args.steps):
        for m in range(len(MAPS)):
            h_outs[m].copy_(outs[m], non_blocking=True)
    barrier()
    d2h_ms = 1e3 * (time.perf_counter() - t0) / args.steps
    del d_tmp

    total_halos = N * ws
    value = job_throughput(N, ws, ms)
    upd = st["hp_updates"] * len(MAPS)
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except Exception:
        pass
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    # roofline of the dominant phase, the HEALPix paint (k_paint_halos, the fused
    # enumerate-and-paint kernel, ~90% of it, and k_paint_full for the large halos on a side
    # stream), timed by CUDA events on the paint stream from before the two launches to
    # their join.  Algorithmic bytes per launch, the per-unit figure of the two-float
    # accumulator: 16 B per pixel update and map (read-modify-write of hi + lo), U = pixel
    # updates summed over the maps.
    paint_ms = phases["paint"]
    alg_paint = upd * 16
    achieved = alg_paint / (paint_ms * 1e-3) / 1e9 if paint_ms > 0 else None
    # DRAM traffic of the paint from the ncu capture of this workload's launch, per pixel
    # update processed
    traffic = PAINT_DRAM_BYTES_PER_UPDATE * st["hp_updates"] if args.precision == "mixed" else None
    roof = {"bound": "hbm", "kernel": "k_paint_halos + k_paint_full", "achieved": achieved,
            "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak if achieved else None,
            "peak_source": ("measured (MEASURED_PEAKS.json hbm_gbs)" if peak_src == "measured"
                            else "fallback 6.8 TB/s"),
            "traffic": traffic, "algorithmic_bytes": alg_paint, "launch_ms": paint_ms,
            "atomic_updates_per_s": upd / (paint_ms * 1e-3) if paint_ms > 0 else None,
            "atomic_peak_per_s": L2_ATOMIC_SECTORS_PER_S,
            "atomic_frac": upd / (paint_ms * 1e-3) / L2_ATOMIC_SECTORS_PER_S if paint_ms > 0 else None}
    # The DRAM floor of a scatter by atomics, in any painting order: every part of the
    # maps that the paint touches is read from DRAM once and written back once.  Counted
    # from the maps of the last resident step (the parts holding a nonzero value): reads
    # of the touched 64-byte blocks, write-back of the touched 32-byte sectors.  The low
    # words' sectors and the halo records come on top.
    if npix % 16 == 0 and paint_ms > 0:
        sec = sum(int(o.view(-1, 8).ne(0).any(dim=1).sum()) for o in outs)
        blk = sum(int(o.view(-1, 16).ne(0).any(dim=1).sum()) for o in outs)
        floor = blk * 64 + sec * 32
        roof["sector_floor"] = {"touched_sectors_32b": sec, "touched_blocks_64b": blk,
                                "bytes": floor, "bytes_per_update": floor / upd,
                                "achieved_gbs": floor / (paint_ms * 1e-3) / 1e9,
                                "frac": floor / (paint_ms * 1e-3) / 1e9 / hbm_peak}
    # the whole step (ingest through maps ready): the algorithmic bytes of the path with a
    # two-float accumulator (catalogue read, 16 B per update, accumulator zero-fill + read
    # and output write per pixel and map), and the bytes no design can avoid (catalogue
    # read once, both float maps written once)
    step_alg = N * 40 + upd * 16 + len(MAPS) * npix * (8 + 4)
    step_min = N * 40 + len(MAPS) * npix * 4
    step_roof = {"algorithmic_bytes": step_alg,
                 "achieved_gbs": step_alg / (ms * 1e-3) / 1e9,
                 "frac": step_alg / (ms * 1e-3) / 1e9 / hbm_peak,
                 "min_bytes": step_min,
                 "min_frac": step_min / (ms * 1e-3) / 1e9 / hbm_peak}

    out = {"metric": METRIC, "value": value, "unit": "halos/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (Philox catalogue, seed %d; profile table from make_maptable "
                   "on the GPU)" % SEED,
           "config": {"workload": workload_name(N, nside),
                      "precision": args.precision, "l2": "inputs and maps larger than L2",
                      "tuning": tunings.get(args.precision),
                      "parallelism": "replicas" if ws > 1 else "single GPU"},
           "pixel_updates_per_s": upd * ws / (ms * 1e-3),
           "phases_ms": phases,
           "counts": {k: st[k] for k in ("n_shell", "n_painted", "n_enumerated",
                                          "hp_candidates", "hp_updates", "n_recheck")},
           "gpu_launches": None,
           "roofline": roof,
           "step_roofline": step_roof,
           "clocks": clocks,
           "e2e": {"value": total_halos / (e2e_ms * 1e-3), "unit": "halos/s",
                   "ms_per_step": e2e_ms, "h2d_bytes_per_step": int(rec.nbytes),
                   "d2h_bytes_per_step": int(len(MAPS) * npix * 4),
                   "h2d_ms": h2d_ms, "d2h_ms": d2h_ms,
                   "pipelined": "step k's map read-back (p2m_get_healpix_async) overlaps "
                                "step k+1's catalogue copy and paint into alternate buffers",
                   "sequential": {"value": total_halos / (e2e_seq_ms * 1e-3),
                                  "ms_per_step": e2e_seq_ms},
                   "maps_vs_resident_max_rel": e2e_check}}
    # per step: the fused cut and set-up, the item kernel of the large halos, their
    # candidate counts and 3-kernel scan, the painting order's 3-kernel scan and scatter,
    # the fused paint, the large-halo paint, the fold of the low words, and the two
    # counter read-outs (memsets are not kernels)
    out["gpu_launches"] = LAUNCHES_PER_STEP * args.steps

    plain_maps = None
    if not args.no_plain and args.precision == "mixed":
        pp = make("fp64")
        ms64, _ = timed(pp, max(2, args.steps // 2), 1)
        ref_maps = [o.cpu().numpy() for o in outs]
        plain_maps = ref_maps
        phases64 = pp.timings()
        pp.close()
        out["plain_fp64"] = {"value": total_halos / (ms64 * 1e-3), "ms_per_step": ms64,
                             "speedup_of_mixed": ms64 / ms, "phases_ms": phases64,
                             "tuning": tunings.get("fp64")}
        errs = {}
        for m, name in enumerate(("tsz", "ksz")):
            errs[name] = map_errors(maps_main[m], ref_maps[m])
            if args.cl_lmax > 0:
                spec = p2m.cl_healpix(maps_main[m], ref_maps[m], lmax=args.cl_lmax, device=local)
                errs[name]["cl_ratio"] = dict(cl_ratio(spec), lmax=args.cl_lmax)
        out["error_vs_fp64"] = errs

        # the deterministic arm: 64-bit fixed-point accumulation; its maps are compared bit
        # for bit with a second run whose launch parameters send every halo through the
        # other painting kernel (so the atomics land in another order)
        pf = make("fixed")
        msf, _ = timed(pf, max(2, args.steps // 2), 1)
        fixed_maps = [o.cpu().numpy() for o in outs]
        pf.close()
        pf = p2m.Painter(nside=nside, precision="fixed", maps=MAPS, zmax=ZMAX, max_records=N,
                         device=local)
        pf.load_table(0, table)
        pf.set_tuning(big_rings=0)
        pf.paint_records_device(d_rec.data_ptr(), N, 10)
        other = [pf.healpix(m) for m in range(len(MAPS))]
        pf.close()
        out["fixed_point"] = {
            "value": total_halos / (msf * 1e-3), "ms_per_step": msf,
            "bit_identical_across_launch_parameters": all(
                np.array_equal(a.view(np.uint32), b.view(np.uint32))
                for a, b in zip(fixed_maps, other)),
            "tuning": tunings.get("fixed"),
            "error_vs_fp64": {name: map_errors(fixed_maps[m], ref_maps[m])
                              for m, name in enumerate(("tsz", "ksz"))}}

    if rank == 0 and ws == 1 and not args.no_files:
        out["e2e_files"] = e2e_files(rec, table, nside, args.precision)

    # the other configurations' reports run in single-GPU runs only (replica runs time
    # the headline workload alone)
    if rank == 0 and ws == 1 and not args.no_precision_form:
        out["precision_form"] = precision_form(local)
    if rank == 0 and ws == 1 and not args.no_ensemble:
        out["ensemble"] = ensemble_form(local)
    if rank == 0 and ws == 1 and not args.no_multi_table:
        out["multi_table"] = multi_table_form(local)

    # the cpu_baseline leg: the oracle timed as the CPU implementation of the path, and
    # the oracle as the checker of this run's maps
    if rank == 0 and ws == 1 and not args.no_cpu:
        times, info = cpu_reference(rec, nside, os.cpu_count() or 1, table, 3, 1)
        out["cpu_baseline"] = dict(info, value=N / float(np.median(times)))
        if not args.no_parity:
            out["parity_vs_oracle"] = parity_vs_oracle(rec, table, nside, maps_main,
                                                       plain_maps, local)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
