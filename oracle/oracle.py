"""ctypes front-end of the oracle (oracle/spirit_oracle.c).

TEST INFRASTRUCTURE ONLY: results are compared against it.  tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg import this module; the product package never does.

The oracle is a CPU FP64 restatement of the reference's hot path (Spirit v2.2.0:
core/src/engine/Hamiltonian_Heisenberg.cpp, Neighbours.cpp, Method_LLG.cpp, Method_GNEB.cpp,
core/include/engine/Solver_*.hpp); its parity with the reference is pinned by the golden
fixtures in tests/golden/.  A system is described by the same "spec" dictionary that
spirit_gb300.configs.write_config() turns into a reference config file.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle_spirit.so")

_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(
            os.path.join(HERE, "spirit_oracle.c")
        ):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.POINTER
        d, i, vp = ctypes.c_double, ctypes.c_int, ctypes.c_void_p
        L.og_create.restype = vp
        L.og_create.argtypes = [P(i), i, P(d), P(d), d, P(d), P(i)]
        L.og_free.argtypes = [vp]
        L.og_nos.argtypes = [vp]
        L.og_positions.argtypes = [vp, P(d)]
        L.og_set_threads.argtypes = [i]
        L.og_set_field.argtypes = [vp, d, P(d)]
        L.og_set_anisotropy.argtypes = [vp, i, P(i), P(d), P(d)]
        L.og_set_exchange_shells.argtypes = [vp, i, P(d)]
        L.og_set_dmi_shells.argtypes = [vp, i, P(d), i]
        L.og_set_exchange_pairs.argtypes = [vp, i, P(i), P(d)]
        L.og_set_dmi_pairs.argtypes = [vp, i, P(i), P(d), P(d)]
        L.og_set_ddi.argtypes = [vp, i, P(i), d, i]
        L.og_n_exchange_pairs.argtypes = [vp]
        L.og_n_dmi_pairs.argtypes = [vp]
        L.og_get_exchange_pairs.argtypes = [vp, P(i), P(d)]
        L.og_get_dmi_pairs.argtypes = [vp, P(i), P(d), P(d)]
        L.og_idx_from_pair.argtypes = [vp, i, P(i)]
        L.og_gradient.argtypes = [vp, P(d), P(d)]
        L.og_gradient_and_energy.argtypes = [vp, P(d), P(d)]
        L.og_gradient_and_energy.restype = d
        L.og_energy_contributions.argtypes = [vp, P(d), P(d), ctypes.c_char_p, i]
        L.og_energy.argtypes = [vp, P(d)]
        L.og_energy.restype = d
        L.og_gradient_ddi_direct.argtypes = [vp, P(d), P(d)]
        L.og_thermal_noise.argtypes = [vp, d, d, d, ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, P(d)]
        L.og_philox4x32.argtypes = [P(ctypes.c_uint32), P(ctypes.c_uint32), P(ctypes.c_uint32)]
        L.og_llg_run.argtypes = [vp, vp, i, i, P(d), P(d), P(d)]
        L.og_gneb_run.argtypes = [vp, vp, i, i, P(d), P(i), P(d), P(d), P(d)]
        L.og_gneb_run_solver.argtypes = [vp, vp, i, i, i, P(d), P(i), P(d), P(d), P(d)]
        L.og_htst.argtypes = [vp, P(d), P(d), i, i, vp, P(d), P(d), P(d), P(d), P(d)]
        L.og_htst.restype = i
        L.og_mc_colors.argtypes = [vp, P(i)]
        L.og_mc_colors.restype = i
        L.og_mc_run.argtypes = [vp, vp, i, P(d), P(d), P(d)]
        L.og_mc_run.restype = i
        L.og_gneb_image_types_auto.argtypes = [i, P(d), P(i)]
        L.og_transition_homogeneous.argtypes = [i, i, P(d), i, i]
        _lib = L
    return _lib


def _p(a, ct=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(ct))


class LLGParams(ctypes.Structure):
    _fields_ = [
        ("dt", ctypes.c_double),
        ("damping", ctypes.c_double),
        ("temperature", ctypes.c_double),
        ("direct_minimization", ctypes.c_int),
        ("force_convergence", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("stream", ctypes.c_uint32),
    ]


class GNEBParams(ctypes.Structure):
    _fields_ = [
        ("spring_constant", ctypes.c_double),
        ("force_convergence", ctypes.c_double),
        ("dt", ctypes.c_double),
    ]


class MCParams(ctypes.Structure):
    _fields_ = [
        ("temperature", ctypes.c_double),
        ("cone", ctypes.c_int),
        ("cone_angle_deg", ctypes.c_double),
        ("adaptive", ctypes.c_int),
        ("acceptance_target", ctypes.c_double),
        ("seed", ctypes.c_uint64),
        ("stream", ctypes.c_uint32),
    ]


BRAVAIS = {
    # core/src/data/Geometry.cpp:446-487
    "sc": [[1, 0, 0], [0, 1, 0], [0, 0, 1]],
    "fcc": [[0.5, 0.0, 0.5], [0.5, 0.5, 0.0], [0.0, 0.5, 0.5]],
    "bcc": [[0.5, 0.5, -0.5], [-0.5, 0.5, -0.5], [0.5, -0.5, -0.5]],
    "hex2d": [[0.5 * np.sqrt(3), -0.5, 0], [0.5 * np.sqrt(3), 0.5, 0], [0, 0, 1]],
    "hex2d60": [[0.5 * np.sqrt(3), -0.5, 0], [0.5 * np.sqrt(3), 0.5, 0], [0, 0, 1]],
    "hex2d120": [[0.5, -0.5 * np.sqrt(3), 0], [0.5, 0.5 * np.sqrt(3), 0], [0, 0, 1]],
}

SOLVER = {"VP": 0, "SIB": 1, "Depondt": 2, "Heun": 3, "RK4": 4, "LBFGS_OSO": 5, "VP_OSO": 7}


def bravais_of(spec):
    if "bravais_vectors" in spec:
        return np.asarray(spec["bravais_vectors"], dtype=np.float64)
    return np.asarray(BRAVAIS[spec.get("bravais", "sc")], dtype=np.float64)


def _normalized(v):
    v = np.asarray(v, dtype=np.float64)
    n = np.sqrt(v @ v)
    return v / n if n > 0 else v


class OracleSystem:
    """One spin system of the oracle, built from a spec dictionary (see spirit_gb300.configs)."""

    def __init__(self, spec):
        L = lib()
        self.spec = spec
        basis = np.asarray(spec.get("basis", [[0, 0, 0]]), dtype=np.float64)
        nb = basis.shape[0]
        mu = np.asarray(spec.get("mu_s", [1.0]), dtype=np.float64)
        if mu.size < nb:
            mu = np.concatenate([mu, np.full(nb - mu.size, mu[0])])
        ncells = np.asarray(spec["n_cells"], dtype=np.int32)
        bc = np.asarray(spec.get("bc", [0, 0, 0]), dtype=np.int32)
        brav = np.ascontiguousarray(bravais_of(spec))
        self.h = L.og_create(
            _p(ncells, ctypes.c_int), nb, _p(brav), _p(np.ascontiguousarray(basis)),
            float(spec.get("lattice_constant", 1.0)), _p(mu), _p(bc, ctypes.c_int),
        )
        if not self.h:
            raise ValueError("oracle: invalid geometry")
        self.nos = L.og_nos(self.h)
        B, Bn = spec.get("field", (0.0, (0, 0, 1)))
        Bn = _normalized(Bn) if np.linalg.norm(Bn) >= 1e-8 else np.array([0, 0, 1.0])
        L.og_set_field(self.h, float(B), _p(np.ascontiguousarray(Bn)))
        K, Kn = spec.get("anisotropy", (0.0, (0, 0, 1)))
        if K != 0:
            idx = np.arange(nb, dtype=np.int32)
            mag = np.full(nb, float(K))
            nrm = np.tile(_normalized(Kn), (nb, 1))
            L.og_set_anisotropy(self.h, nb, _p(idx, ctypes.c_int), _p(mag), _p(np.ascontiguousarray(nrm)))
        if spec.get("pairs") is not None:
            self._set_pairs(spec["pairs"])
        else:
            jij = np.asarray(spec.get("jij", []), dtype=np.float64)
            dij = np.asarray(spec.get("dij", []), dtype=np.float64)
            if jij.size:
                L.og_set_exchange_shells(self.h, jij.size, _p(jij))
            if dij.size:
                L.og_set_dmi_shells(self.h, dij.size, _p(dij), int(spec.get("dm_chirality", 1)))
        ddi = spec.get("ddi")
        if ddi:
            method = {"none": 0, "fft": 1, "cutoff": 3}[ddi.get("method", "fft")]
            img = np.asarray(ddi.get("n_periodic_images", [4, 4, 4]), dtype=np.int32)
            L.og_set_ddi(self.h, method, _p(img, ctypes.c_int), float(ddi.get("radius", 0.0)),
                         int(ddi.get("pb_zero_padding", 1)))

    def _set_pairs(self, rows):
        # explicit pair table (i j da db dc Jij Dijx Dijy Dijz): Dataparser.cpp Pairs_from_File
        ex, exJ, dm, dmD, dmN = [], [], [], [], []
        for r in rows:
            i, j, da, db, dc, J, dx, dy, dz = r
            key = (i, j, da, db, dc)
            if J != 0:
                for k, q in enumerate(ex):
                    if q == key or (q[0] == j and q[1] == i and (q[2], q[3], q[4]) == (-da, -db, -dc)):
                        exJ[k] += J
                        break
                else:
                    ex.append(key)
                    exJ.append(J)
            dn = np.sqrt(dx * dx + dy * dy + dz * dz)
            if dn != 0:
                dm.append(key)
                dmD.append(dn)
                dmN.append([dx / dn, dy / dn, dz / dn])
        L = lib()
        if ex:
            a = np.asarray(ex, dtype=np.int32)
            L.og_set_exchange_pairs(self.h, len(ex), _p(a, ctypes.c_int), _p(np.asarray(exJ, dtype=np.float64)))
        if dm:
            a = np.asarray(dm, dtype=np.int32)
            L.og_set_dmi_pairs(self.h, len(dm), _p(a, ctypes.c_int), _p(np.asarray(dmD, dtype=np.float64)),
                               _p(np.ascontiguousarray(np.asarray(dmN, dtype=np.float64))))

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.og_free(self.h)
            self.h = None

    # -- geometry / pairs
    def positions(self):
        out = np.zeros((self.nos, 3))
        lib().og_positions(self.h, _p(out))
        return out

    def exchange_pairs(self):
        n = lib().og_n_exchange_pairs(self.h)
        pairs = np.zeros((n, 5), dtype=np.int32)
        mag = np.zeros(n)
        lib().og_get_exchange_pairs(self.h, _p(pairs, ctypes.c_int), _p(mag))
        return pairs, mag

    def dmi_pairs(self):
        n = lib().og_n_dmi_pairs(self.h)
        pairs = np.zeros((n, 5), dtype=np.int32)
        mag = np.zeros(n)
        nrm = np.zeros((n, 3))
        lib().og_get_dmi_pairs(self.h, _p(pairs, ctypes.c_int), _p(mag), _p(nrm))
        return pairs, mag, nrm

    # -- Hamiltonian
    def gradient(self, spins):
        s = np.ascontiguousarray(spins, dtype=np.float64)
        g = np.zeros_like(s)
        lib().og_gradient(self.h, _p(s), _p(g))
        return g

    def gradient_and_energy(self, spins):
        s = np.ascontiguousarray(spins, dtype=np.float64)
        g = np.zeros_like(s)
        E = lib().og_gradient_and_energy(self.h, _p(s), _p(g))
        return g, E

    def energy_contributions(self, spins):
        s = np.ascontiguousarray(spins, dtype=np.float64)
        out = np.zeros((6, self.nos))
        names = ctypes.create_string_buffer(256)
        n = lib().og_energy_contributions(self.h, _p(s), _p(out), names, 256)
        keys = names.value.decode().split(",") if n else []
        return {k: out[t].copy() for t, k in enumerate(keys)}

    def energy(self, spins):
        s = np.ascontiguousarray(spins, dtype=np.float64)
        return lib().og_energy(self.h, _p(s))

    def gradient_ddi_direct(self, spins):
        s = np.ascontiguousarray(spins, dtype=np.float64)
        g = np.zeros_like(s)
        lib().og_gradient_ddi_direct(self.h, _p(s), _p(g))
        return g

    def thermal_noise(self, temperature, damping, dt, seed, stream, iteration):
        xi = np.zeros((self.nos, 3))
        lib().og_thermal_noise(self.h, temperature, damping, dt, seed, stream, iteration, _p(xi))
        return xi

    # -- methods
    def llg(self, spins, solver, n_iter, dt=1e-3, damping=0.3, temperature=0.0, seed=2006, stream=0,
            direct_minimization=False, force_convergence=1e-10):
        s = np.ascontiguousarray(spins, dtype=np.float64).copy()
        p = LLGParams(dt, damping, temperature, int(direct_minimization), force_convergence, seed, stream)
        E = ctypes.c_double()
        mt = ctypes.c_double()
        solver_id = SOLVER[solver] if isinstance(solver, str) else int(solver)
        it = lib().og_llg_run(self.h, ctypes.byref(p), solver_id, int(n_iter), _p(s), ctypes.byref(E),
                              ctypes.byref(mt))
        return s, {"iterations": it, "energy": E.value, "max_torque": mt.value}

    def mc_colors(self):
        """Greedy colouring of the interaction graph (the Monte Carlo sweep order)."""
        c = np.zeros(self.nos, dtype=np.int32)
        n = lib().og_mc_colors(self.h, _p(c, ctypes.c_int))
        return c, n

    def mc(self, spins, n_sweeps, temperature=0.0, cone=True, cone_angle=30.0, adaptive=True, target=0.5,
           seed=2006, stream=0):
        """Metropolis sweeps (Method_MC with colour-ordered sweeps and Philox draws); returns
        (spins, {"cone_angle": deg, "acceptance": ratio})."""
        s = np.ascontiguousarray(spins, dtype=np.float64).copy()
        p = MCParams(temperature, int(cone), cone_angle, int(adaptive), target, seed, stream)
        ca, ac = ctypes.c_double(), ctypes.c_double()
        lib().og_mc_run(self.h, ctypes.byref(p), int(n_sweeps), _p(s), ctypes.byref(ca), ctypes.byref(ac))
        return s, {"cone_angle": ca.value, "acceptance": ac.value}

    def htst(self, spins_min, spins_sp, sparse=False, n_keep=-1):
        """HTST prefactor of the transition minimum -> saddle point (HTST_Calculate); dict of the
        HTST_Info fields (+ eigenvalues / eigenvectors [mode][2N] / velocities when dense)."""
        return _htst(self, spins_min, spins_sp, sparse, n_keep)

    def gneb(self, chain, n_iter, image_type=None, spring_constant=1.0, force_convergence=1e-6, dt=1e-3,
             solver="VP"):
        c = np.ascontiguousarray(chain, dtype=np.float64).copy()
        noi = c.shape[0]
        types = np.zeros(noi, dtype=np.int32) if image_type is None else np.asarray(image_type, dtype=np.int32)
        E = np.zeros(noi)
        Rx = np.zeros(noi)
        mt = ctypes.c_double()
        p = GNEBParams(spring_constant, force_convergence, dt)
        solver_id = SOLVER[solver] if isinstance(solver, str) else int(solver)
        it = lib().og_gneb_run_solver(self.h, ctypes.byref(p), solver_id, noi, int(n_iter), _p(c),
                                      _p(types, ctypes.c_int), _p(E), _p(Rx), ctypes.byref(mt))
        return c, {"iterations": it, "energies": E, "Rx": Rx, "max_torque": mt.value}


class HTSTInfo(ctypes.Structure):
    _fields_ = [(k, ctypes.c_double) for k in ("temperature_exponent", "me", "Omega_0", "s", "volume_min",
                                               "volume_sp", "prefactor_dynamical", "prefactor", "det_min",
                                               "det_sp")] + [("n_eigenmodes_keep", ctypes.c_int),
                                                             ("status", ctypes.c_int)]


def _htst(system, spins_min, spins_sp, sparse=False, n_keep=-1):
    nos = system.nos
    a = np.ascontiguousarray(spins_min, dtype=np.float64)
    b = np.ascontiguousarray(spins_sp, dtype=np.float64)
    n2 = 2 * nos
    keep = n2 if n_keep < 0 else min(n_keep, n2)
    em, es = np.zeros(n2), np.zeros(n2)
    vm, vs = np.zeros((max(keep, 1), n2)), np.zeros((max(keep, 1), n2))
    vel = np.zeros(n2)
    info = HTSTInfo()
    lib().og_htst(system.h, _p(a), _p(b), int(sparse), int(n_keep), ctypes.byref(info), _p(em), _p(es), _p(vm),
                  _p(vs), _p(vel))
    out = {k: getattr(info, k) for k, _ in HTSTInfo._fields_}
    if not sparse:
        out.update(evalues_min=em, evalues_sp=es, evectors_min=vm[:keep], evectors_sp=vs[:keep], velocities=vel)
    return out


def image_types_auto(energies, image_type):
    t = np.ascontiguousarray(image_type, dtype=np.int32).copy()
    e = np.ascontiguousarray(energies, dtype=np.float64)
    lib().og_gneb_image_types_auto(len(e), _p(e), _p(t, ctypes.c_int))
    return t


def transition_homogeneous(chain, idx_1, idx_2):
    c = np.ascontiguousarray(chain, dtype=np.float64).copy()
    lib().og_transition_homogeneous(c.shape[1], c.shape[0], _p(c), idx_1, idx_2)
    return c


def philox4x32(ctr, key):
    c = np.asarray(ctr, dtype=np.uint32)
    k = np.asarray(key, dtype=np.uint32)
    o = np.zeros(4, dtype=np.uint32)
    lib().og_philox4x32(_p(c, ctypes.c_uint32), _p(k, ctypes.c_uint32), _p(o, ctypes.c_uint32))
    return o


def portable_spins(nos, seed):
    """Uniform directions on S^2 that come out bit-identical on every platform: points drawn
    uniformly in the cube [-1, 1]^3 by numpy's legacy MT19937 RandomState (a stream numpy keeps
    frozen), those outside the unit ball or too close to the origin rejected, the rest scaled by
    1 / |v| -- only additions, multiplications, division and square root (all correctly rounded),
    no platform libm.  The inputs of the full-size fixtures are regenerated from their seed on any
    machine."""
    rs = np.random.RandomState(seed)
    out = np.empty((0, 3))
    while len(out) < nos:
        v = rs.uniform(-1.0, 1.0, (2 * (nos - len(out)) + 16, 3))
        r2 = (v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1]) + v[:, 2] * v[:, 2]
        v = v[(r2 <= 1.0) & (r2 >= 0.01)]
        out = np.concatenate([out, v])
    out = out[:nos]
    n = np.sqrt((out[:, 0] * out[:, 0] + out[:, 1] * out[:, 1]) + out[:, 2] * out[:, 2])
    return np.ascontiguousarray(out / n[:, None])


def random_spins(nos, seed):
    """Uniform directions on S^2 (z in U[-1,1], phi in U[-pi,pi], as Vectormath.cpp:41-51)."""
    rng = np.random.default_rng(seed)
    z = rng.uniform(-1.0, 1.0, nos)
    phi = rng.uniform(-np.pi, np.pi, nos)
    r = np.sqrt(1 - z * z)
    return np.ascontiguousarray(np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1))
