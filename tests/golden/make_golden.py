"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Runs oracle/_ref/golden_harness (the reference, Spirit v2.2.0, CPU/OpenMP FP64 with kissFFT,
compiled from its sources by oracle/ref/Makefile) on the cases of cases.py, with input spins
generated here from fixed seeds and injected through System_Get_Spin_Directions, and packs
its outputs into small .npz files.  Needs the reference sources (only in the build
container); the fixtures it writes are committed and the tests read only those.

    make -C oracle/ref -j8 && python tests/golden/make_golden.py [--only SUBSTRING]

--only regenerates just the fixtures whose name contains SUBSTRING.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from cases import (FULL_CASES, GRAD_CASES, HTST_CASES, LLG_CASES, OVF_FORMATS, OVF_SPEC, PAIR_GEOMETRIES,  # noqa: E402
                   SOLVERS, SPIN_SEED, THERMAL_CASES)
from oracle.oracle import (OracleSystem, image_types_auto, portable_spins, random_spins,  # noqa: E402
                           transition_homogeneous)
from spirit_gb300.configs import config_text, write_config  # noqa: E402

HARNESS = os.path.join(ROOT, "oracle", "_ref", "golden_harness")
HTST_KEYS = ["temperature_exponent", "me", "Omega_0", "s", "volume_min", "volume_sp", "prefactor_dynamical",
             "prefactor", "det_min", "det_sp"]


def run(args, cwd, threads=4):
    r = subprocess.run([HARNESS] + args, cwd=cwd, capture_output=True, text=True,
                       env=dict(os.environ, OMP_NUM_THREADS=str(threads)))
    if r.returncode != 0:
        raise RuntimeError("harness failed: %s\n%s" % (args, r.stderr[-2000:]))


def load_bin(path, shape=None):
    a = np.fromfile(path, dtype=np.float64)
    return a.reshape(shape) if shape is not None else a


def load_kv(path):
    out = {}
    for line in open(path):
        k, v = line.split()[:2]
        out[k] = float(v)
    return out


def nos_of(spec):
    n = spec["n_cells"]
    return n[0] * n[1] * n[2] * len(spec.get("basis", [[0, 0, 0]]))


def main(only=None):
    tmp = tempfile.mkdtemp(prefix="golden_")
    out = {}

    def want(tag):
        return only is None or only in tag

    # --- neighbour / DMI pair lists
    for name, spec in PAIR_GEOMETRIES.items():
        if not want("pairs_" + name):
            continue
        cfg = write_config(spec, os.path.join(tmp, name + ".cfg"))
        run(["pairs", cfg, os.path.join(tmp, name)], tmp)
        ex = np.loadtxt(os.path.join(tmp, name + "_exchange.txt"), ndmin=2)
        dm = np.loadtxt(os.path.join(tmp, name + "_dmi.txt"), ndmin=2)
        np.savez_compressed(
            os.path.join(HERE, "pairs_%s.npz" % name), config=config_text(spec),
            exchange_pairs=ex[:, :5].astype(np.int32), exchange_magnitudes=ex[:, 5],
            dmi_pairs=dm[:, :5].astype(np.int32), dmi_magnitudes=dm[:, 5], dmi_normals=dm[:, 6:9],
            positions=load_bin(os.path.join(tmp, name + "_positions.bin"), (-1, 3)),
        )
        out[name] = (len(ex), len(dm))
    # --- gradients and energies
    for name, spec in GRAD_CASES.items():
        if not want("grad_" + name):
            continue
        cfg = write_config(spec, os.path.join(tmp, name + ".cfg"))
        nos = nos_of(spec)
        spins = random_spins(nos, SPIN_SEED[name])
        sp = os.path.join(tmp, name + "_spins.bin")
        spins.tofile(sp)
        run(["grad", cfg, sp, os.path.join(tmp, name)], tmp)
        E = load_kv(os.path.join(tmp, name + "_energy.txt"))
        terms = {k: v for k, v in E.items() if k not in ("grad_and_energy", "total")}
        per_spin = {"energy_" + k: load_bin(os.path.join(tmp, "%s_energy_%s.bin" % (name, k))) for k in terms}
        extra = {}
        if spec.get("ddi"):
            run(["direct", cfg, sp, os.path.join(tmp, name + "_direct")], tmp)
            extra["gradient_direct"] = load_bin(os.path.join(tmp, name + "_direct_gradient.bin"), (-1, 3))
            Ed = load_kv(os.path.join(tmp, name + "_direct_energy.txt"))
            extra["energy_direct"] = Ed["total"]
        np.savez_compressed(
            os.path.join(HERE, "grad_%s.npz" % name), config=config_text(spec), spins=spins,
            gradient=load_bin(os.path.join(tmp, name + "_gradient.bin"), (-1, 3)),
            gradient_ge=load_bin(os.path.join(tmp, name + "_grad_and_energy_gradient.bin"), (-1, 3)),
            energy_ge=E["grad_and_energy"], energy_total=E["total"],
            term_names=np.array(list(terms.keys())), term_energies=np.array(list(terms.values())),
            **per_spin, **extra,
        )
        out[name] = E["total"]
    # --- LLG trajectories (T = 0)
    for case, sname, sid, n_iter in LLG_CASES:
        if not want("llg_%s_%s" % (case, sname)):
            continue
        spec = GRAD_CASES[case]
        cfg = write_config(spec, os.path.join(tmp, case + ".cfg"))
        nos = nos_of(spec)
        spins = random_spins(nos, SPIN_SEED[case] + 100)
        sp = os.path.join(tmp, case + "_llg_spins.bin")
        spins.tofile(sp)
        tag = os.path.join(tmp, "llg_%s_%s" % (case, sname))
        run(["llg", cfg, sp, tag, str(sid), str(n_iter)], tmp)
        res = load_kv(tag + "_result.txt")
        np.savez_compressed(
            os.path.join(HERE, "llg_%s_%s.npz" % (case, sname)), config=config_text(spec), spins_in=spins,
            spins_out=load_bin(tag + "_spins.bin", (-1, 3)), solver=sid, n_iter=n_iter,
            energy=res["energy_image"], max_torque=res["max_torque"], iterations=int(res["iterations"]),
        )
        out["llg_%s_%s" % (case, sname)] = res
    # --- the benchmark configurations at full size (T = 0).  The dipolar system runs on one thread:
    # the reference's kissFFT path slows down with more OpenMP threads.  Outputs of the large
    # system are kept as FP32 (the device FP32 bar is 1e-5) plus every 16th spin in FP64 (pins the
    # oracle to rounding) and the FP64 energy; inputs are regenerated from the seed (portable_spins)
    # and checked against the stored sums.
    for name, spec, sname, sid, n_iter, seed in FULL_CASES:
        if not want("full_" + name):
            continue
        cfg = write_config(spec, os.path.join(tmp, name + ".cfg"))
        nos = nos_of(spec)
        spins = portable_spins(nos, seed)
        sp = os.path.join(tmp, name + "_spins.bin")
        spins.tofile(sp)
        tag = os.path.join(tmp, "full_" + name)
        run(["llg", cfg, sp, tag, str(sid), str(n_iter)], tmp, threads=1 if spec.get("ddi") else 4)
        res = load_kv(tag + "_result.txt")
        so = load_bin(tag + "_spins.bin", (-1, 3))
        big = nos > 65536
        np.savez_compressed(
            os.path.join(HERE, "full_%s.npz" % name), config=config_text(spec), seed=seed, solver=sid,
            n_iter=n_iter, spins_in_sum=spins.sum(axis=0), spins_in_head=spins[:64],
            spins_out=so.astype(np.float32) if big else so, spins_out_fp64_every16=so[::16],
            energy=res["energy_image"], max_torque=res["max_torque"], iterations=int(res["iterations"]),
        )
        out["full_" + name] = res
    # --- OVF interchange: the reference writes the seeded spins in every format (files committed
    # under ovf/), and reads back files this library wrote (what it read is stored)
    if want("ovf"):
        from spirit_gb300 import io as sio
        from spirit_gb300 import state as sstate
        from spirit_gb300 import system as ssystem

        odir = os.path.join(HERE, "ovf")
        os.makedirs(odir, exist_ok=True)
        cfg = write_config(OVF_SPEC, os.path.join(tmp, "ovf.cfg"))
        nos = nos_of(OVF_SPEC)
        spins = random_spins(nos, 31)
        sp = os.path.join(tmp, "ovf_spins.bin")
        spins.tofile(sp)
        read_back = {}
        for name, fid in OVF_FORMATS.items():
            run(["ovfwrite", cfg, sp, os.path.join(odir, "reference_%s.ovf" % name), str(fid)], tmp)
            ours = os.path.join(odir, "spirit_gb300_%s.ovf" % name)
            with sstate.State(cfg, True) as p:
                ssystem.get_spin_directions(p)[:] = spins
                sio.image_write(p, ours, fid, "written by spirit_gb300")
            out_bin = os.path.join(tmp, "read_%s.bin" % name)
            run(["ovfread", cfg, ours, out_bin], tmp)
            read_back[name] = load_bin(out_bin, (-1, 3))
        np.savez_compressed(os.path.join(HERE, "ovf_interchange.npz"), config=config_text(OVF_SPEC), spins=spins,
                            **{"reference_read_" + k: v for k, v in read_back.items()})
        out["ovf"] = sorted(read_back)
    # --- thermal statistics: the reference's own LLG (host mt19937 noise) and Monte Carlo at T > 0;
    # the time series of (E, m) are stored, the statistics are formed by tests/thermal_stats.py
    for name, spec, method, sid, T, n_eq, n_s, stride, start in THERMAL_CASES:
        if not want("thermal_" + name):
            continue
        cfg = write_config(spec, os.path.join(tmp, name + ".cfg"))
        nos = nos_of(spec)
        spins = random_spins(nos, 41) if start == "random" else np.tile([0.0, 0.0, 1.0], (nos, 1))
        sp = os.path.join(tmp, name + "_spins.bin")
        spins.tofile(sp)
        tag = os.path.join(tmp, "thermal_" + name)
        run(["thermal", cfg, sp, tag, method, str(sid), repr(T), str(n_eq), str(n_s), str(stride)], tmp, threads=1)
        ser = load_bin(tag + "_series.bin", (n_s, 4))
        np.savez_compressed(os.path.join(HERE, "thermal_%s.npz" % name), config=config_text(spec), method=method,
                            solver=sid, temperature=T, n_equil=n_eq, n_samples=n_s, stride=stride, start=start,
                            energy=ser[:, 0], m=ser[:, 1:])
        out["thermal_" + name] = (ser[:, 3].mean(), ser[:, 0].mean() / nos)
    # --- the GNEB benchmark chain (32 images of the 96x96 triangular lattice): the oracle relaxes the
    # Neel skyrmion and converges the chain (FP64, climbing image, max torque < 1e-6 meV); the
    # reference continues from that chain for 50 iterations with its own climbing-image types.
    # The chain itself is not stored (7 MB); its barrier and energies are.
    if want("c3_barrier"):
        import bench
        from spirit_gb300.configs import write_config as _wc

        spec = bench.C3_SPEC
        o = OracleSystem(spec)
        pos = o.positions()
        center = 0.5 * (pos.min(axis=0) + pos.max(axis=0))
        sign = min((1.0, -1.0), key=lambda sg: o.energy(bench.neel_skyrmion(pos, center, sign=sg)))
        # the relaxed skyrmion (a local minimum; the device relaxes it with VP, the oracle with L-BFGS)
        sk, r0 = o.llg(bench.neel_skyrmion(pos, center, sign=sign), "LBFGS_OSO", 20000, dt=1e-3,
                       force_convergence=1e-9)
        noi = bench.C3_IMAGES
        chain = np.zeros((noi,) + sk.shape)
        chain[0] = sk
        chain[-1] = [0.0, 0.0, 1.0]
        chain = transition_homogeneous(chain, 0, noi - 1)
        chain, r1 = o.gneb(chain, 2000, spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
        types = image_types_auto(r1["energies"], np.zeros(noi))
        chain, r2 = o.gneb(chain, 200000, image_type=types, spring_constant=1.0, force_convergence=1e-6, dt=1e-3)
        cfg = _wc(spec, os.path.join(tmp, "c3.cfg"))
        cp = os.path.join(tmp, "c3_chain.bin")
        chain.tofile(cp)
        tag = os.path.join(tmp, "c3_ref")
        run(["gneb", cfg, cp, tag, str(noi), "0", "1", "50"], tmp, threads=8)
        rows = [l.split() for l in open(tag + "_result.txt")]
        img = [r_ for r_ in rows if r_[0] == "image"]
        Eref = np.array([float(r_[3]) for r_ in img])
        np.savez_compressed(
            os.path.join(HERE, "gneb_c3_barrier.npz"), config=config_text(spec), skyrmion_sign=sign,
            oracle_energies=r2["energies"], oracle_barrier=float(r2["energies"].max() - r2["energies"][0]),
            oracle_iterations=int(r1["iterations"]) + int(r2["iterations"]), oracle_max_torque=r2["max_torque"],
            reference_energies=Eref, reference_barrier=float(Eref.max() - Eref[0]),
            reference_max_torque=float([r_ for r_ in rows if r_[0] == "max_torque"][0][1]),
            reference_image_type=np.array([int(r_[7]) for r_ in img]), image_type=types,
        )
        out["c3_barrier"] = (r2["energies"].max() - r2["energies"][0], Eref.max() - Eref[0], r2["max_torque"])
    # --- GNEB (VP) on the reference solver-test system: skyrmion collapse, 9 images
    spec = SOLVERS
    cfg = write_config(spec, os.path.join(tmp, "solvers.cfg"))
    nos = nos_of(spec)
    noi = 9
    o = OracleSystem(spec)
    pos = o.positions()
    centre = pos.mean(axis=0)
    r = np.linalg.norm(pos[:, :2] - centre[:2], axis=1)
    theta = np.pi * np.clip(1 - r / 5.0, 0, 1)  # linear-profile skyrmion of radius 5
    phi = np.arctan2(pos[:, 1] - centre[1], pos[:, 0] - centre[0]) + np.pi / 2  # Bloch helicity
    sk = np.stack([np.sin(theta) * np.cos(phi), np.sin(theta) * np.sin(phi), np.cos(theta)], axis=1)
    chain = np.zeros((noi, nos, 3))
    chain[0] = sk
    chain[-1] = np.array([0, 0, 1.0])
    chain = transition_homogeneous(chain, 0, noi - 1)
    cp = os.path.join(tmp, "chain.bin")
    chain.tofile(cp)
    # VP with a chain-global velocity projection switches branches on rounding-level differences,
    # so step-by-step parity is pinned over a short run; the converged run pins the saddle.
    # The OSO solvers (VP_OSO = 7, LBFGS_OSO = 5) are pinned the same way over short runs.
    for tag_name, sid, n1, n2 in (("gneb_vp", 0, 20, 0), ("gneb_vp_ci", 0, 20, 20),
                                  ("gneb_converged", 0, 20000, 200000), ("gneb_vp_oso", 7, 20, 0),
                                  ("gneb_lbfgs_oso", 5, 20, 0), ("gneb_lbfgs_oso_ci", 5, 20, 20)):
        if not want(tag_name):
            continue
        tag = os.path.join(tmp, tag_name)
        run(["gneb", cfg, cp, tag, str(noi), str(sid), str(n1), str(n2)], tmp)
        rows = [l.split() for l in open(tag + "_result.txt")]
        img = [r_ for r_ in rows if r_[0] == "image"]
        np.savez_compressed(
            os.path.join(HERE, "%s.npz" % tag_name), config=config_text(spec), chain_in=chain,
            chain_out=load_bin(tag + "_chain.bin", (noi, nos, 3)),
            energies=np.array([float(r_[3]) for r_ in img]), Rx=np.array([float(r_[5]) for r_ in img]),
            image_type=np.array([int(r_[7]) for r_ in img]), n_iter=n1, n_iter_ci=n2, solver=sid,
            max_torque=float([r_ for r_ in rows if r_[0] == "max_torque"][0][1]),
        )
        out[tag_name] = [float(r_[3]) for r_ in img]
    # --- HTST: converged minimum and saddle point from the oracle's minimisers (LBFGS_OSO, GNEB with
    # climbing image, torque < 1e-11), then the reference's HTST_Calculate (dense and sparse)
    for name, spec, seed in HTST_CASES:
        if not want("htst_" + name):
            continue
        o = OracleSystem(spec)
        nos = o.nos
        rng = np.random.default_rng(seed)
        ends = []
        for sgn in (1.0, -1.0):
            x = np.tile([0.05, 0.0, sgn], (nos, 1)) + 0.05 * rng.normal(size=(nos, 3))
            x /= np.linalg.norm(x, axis=1, keepdims=True)
            ends.append(o.llg(x, "LBFGS_OSO", 20000, force_convergence=1e-12)[0])
        noi = 9
        chain = np.zeros((noi, nos, 3))
        chain[0], chain[-1] = ends
        chain = transition_homogeneous(chain, 0, noi - 1)
        for k in range(1, noi - 1):
            chain[k] += 0.1 * rng.normal(size=(nos, 3))
            chain[k] /= np.linalg.norm(chain[k], axis=1, keepdims=True)
        chain, r = o.gneb(chain, 3000, solver="LBFGS_OSO", force_convergence=1e-11)
        types = image_types_auto(r["energies"], np.zeros(noi))
        chain, r = o.gneb(chain, 100000, image_type=types, solver="VP_OSO", force_convergence=1e-11)
        sp = int(np.argmax(types == 1))
        cfg = write_config(spec, os.path.join(tmp, "htst_%s.cfg" % name))
        cp = os.path.join(tmp, "htst_%s_chain.bin" % name)
        chain.tofile(cp)
        res = {}
        for sparse in (0, 1):
            tag = os.path.join(tmp, "htst_%s_%d" % (name, sparse))
            run(["htst", cfg, cp, tag, str(noi), "0", str(sp), str(sparse), "-1"], tmp)
            res[sparse] = load_kv(tag + "_result.txt")
        tag = os.path.join(tmp, "htst_%s_0" % name)
        n2 = 2 * nos
        # the reference stops (no eigen output) when a check fails, e.g. a higher-order saddle point
        done = os.path.getsize(tag + "_evalues_min.bin") > 0
        ev = (lambda suffix, shape=None: load_bin(tag + suffix, shape)) if done else (lambda suffix, shape=None: np.zeros(0))
        np.savez_compressed(
            os.path.join(HERE, "htst_%s.npz" % name), config=config_text(spec), spins_min=chain[0], spins_sp=chain[sp],
            sp_index=sp, gneb_max_torque=r["max_torque"],
            dense=np.array([res[0][k] for k in HTST_KEYS]), sparse=np.array([res[1][k] for k in HTST_KEYS]),
            keys=np.array(HTST_KEYS),
            completed=done, evalues_min=ev("_evalues_min.bin"), evalues_sp=ev("_evalues_sp.bin"),
            evectors_min=ev("_evectors_min.bin", (n2, n2)), evectors_sp=ev("_evectors_sp.bin", (n2, n2)),
            velocities=ev("_velocities.bin"),
        )
        out["htst_" + name] = (res[0]["prefactor"], res[1]["prefactor"])
    for k, v in out.items():
        print(k, v)


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--only", default=None)
    main(ap.parse_args().only)
