"""Write Spirit input files (the reference's config-file format, core/docs/Input.md) from a dict.

The same "spec" dictionary drives State_Setup() here and the reference's own State_Setup(), so
both sides parse identical text.  Keys:

    bravais            "sc" | "fcc" | "bcc" | "hex2d" | "hex2d60" | "hex2d120"  (or bravais_vectors)
    n_cells            [Na, Nb, Nc]
    basis              [[x, y, z], ...] in units of the Bravais vectors (default one atom at 0)
    lattice_constant   Angstrom
    mu_s               [mu per basis atom] (Bohr magnetons)
    bc                 [0/1, 0/1, 0/1] periodic boundary conditions
    field              (B [T], (nx, ny, nz))
    anisotropy         (K [meV], (nx, ny, nz))
    jij, dij           shell magnitudes [meV]; dm_chirality 1 Bloch, 2 Neel (negatives invert)
    pairs              explicit table rows (i, j, da, db, dc, Jij, Dijx, Dijy, Dijz) -> heisenberg_pairs
    ddi                {"method": "fft"|"cutoff"|"none", "n_periodic_images": [..], "radius": r,
                        "pb_zero_padding": 0/1}
    llg                {"dt", "damping", "temperature", "seed", "force_convergence", "n_iterations"}
    gneb               {"spring_constant", "force_convergence", "n_iterations"}
"""
import numpy as np


def _fmt(x):
    return repr(float(x))


def config_text(spec):
    lines = [
        "log_to_console 0",
        "log_to_file 0",
        "log_console_level 0",
        "save_input_initial 0",
        "save_input_final 0",
        "save_positions_initial 0",
        "save_positions_final 0",
        "save_neighbours_initial 0",
        "save_neighbours_final 0",
        "llg_output_any 0",
        "gneb_output_any 0",
        "mc_output_any 0",
        "mmf_output_any 0",
    ]
    if "bravais_vectors" in spec:
        lines.append("bravais_vectors")
        for v in spec["bravais_vectors"]:
            lines.append(" ".join(_fmt(x) for x in v))
    else:
        lines.append("bravais_lattice " + spec.get("bravais", "sc"))
    lines.append("n_basis_cells " + " ".join(str(int(n)) for n in spec["n_cells"]))
    basis = spec.get("basis")
    if basis is not None and len(basis) > 0 and not (len(basis) == 1 and not np.any(basis[0])):
        lines.append("basis")
        lines.append(str(len(basis)))
        for b in basis:
            lines.append(" ".join(_fmt(x) for x in b))
    lines.append("lattice_constant " + _fmt(spec.get("lattice_constant", 1.0)))
    lines.append("mu_s " + " ".join(_fmt(m) for m in spec.get("mu_s", [1.0])))
    if spec.get("pairs") is not None:
        lines.append("hamiltonian heisenberg_pairs")
    else:
        lines.append("hamiltonian heisenberg_neighbours")
    lines.append("boundary_conditions " + " ".join(str(int(b)) for b in spec.get("bc", [0, 0, 0])))
    B, Bn = spec.get("field", (0.0, (0, 0, 1)))
    lines.append("external_field_magnitude " + _fmt(B))
    lines.append("external_field_normal " + " ".join(_fmt(x) for x in Bn))
    K, Kn = spec.get("anisotropy", (0.0, (0, 0, 1)))
    lines.append("anisotropy_magnitude " + _fmt(K))
    lines.append("anisotropy_normal " + " ".join(_fmt(x) for x in Kn))
    if spec.get("pairs") is not None:
        rows = spec["pairs"]
        lines.append("n_interaction_pairs %d" % len(rows))
        lines.append("i j da db dc Jij Dijx Dijy Dijz")
        for r in rows:
            lines.append("%d %d %d %d %d %s %s %s %s" % (int(r[0]), int(r[1]), int(r[2]), int(r[3]), int(r[4]),
                                                        _fmt(r[5]), _fmt(r[6]), _fmt(r[7]), _fmt(r[8])))
    else:
        jij = list(spec.get("jij", []))
        dij = list(spec.get("dij", []))
        lines.append("n_shells_exchange %d" % len(jij))
        if jij:
            lines.append("jij " + " ".join(_fmt(x) for x in jij))
        lines.append("n_shells_dmi %d" % len(dij))
        if dij:
            lines.append("dij " + " ".join(_fmt(x) for x in dij))
        lines.append("dm_chirality %d" % int(spec.get("dm_chirality", 1)))
    ddi = spec.get("ddi")
    if ddi:
        lines.append("ddi_method " + ddi.get("method", "fft"))
        lines.append("ddi_n_periodic_images " + " ".join(str(int(x)) for x in ddi.get("n_periodic_images", [4, 4, 4])))
        lines.append("ddi_radius " + _fmt(ddi.get("radius", 0.0)))
        lines.append("ddi_pb_zero_padding %d" % int(ddi.get("pb_zero_padding", 1)))
    else:
        lines.append("ddi_method none")
    llg = spec.get("llg", {})
    lines.append("llg_dt " + _fmt(llg.get("dt", 1e-3)))
    lines.append("llg_damping " + _fmt(llg.get("damping", 0.3)))
    lines.append("llg_temperature " + _fmt(llg.get("temperature", 0.0)))
    lines.append("llg_seed %d" % int(llg.get("seed", 2006)))
    lines.append("llg_force_convergence " + _fmt(llg.get("force_convergence", 1e-10)))
    lines.append("llg_n_iterations %d" % int(llg.get("n_iterations", 2000000)))
    lines.append("llg_n_iterations_log %d" % int(llg.get("n_iterations_log", 2000000)))
    lines.append("llg_max_walltime 0:0:0")
    gneb = spec.get("gneb", {})
    lines.append("gneb_spring_constant " + _fmt(gneb.get("spring_constant", 1.0)))
    lines.append("gneb_force_convergence " + _fmt(gneb.get("force_convergence", 1e-7)))
    lines.append("gneb_n_iterations %d" % int(gneb.get("n_iterations", 200000)))
    lines.append("gneb_n_iterations_log %d" % int(gneb.get("n_iterations_log", 200000)))
    lines.append("gneb_max_walltime 0:0:0")
    return "\n".join(lines) + "\n"


def write_config(spec, path):
    with open(path, "w") as f:
        f.write(config_text(spec))
    return path
