"""Extract the reference's own golden vectors for the H.psi path into golden.json.

Run once in a container that holds the reference sources (their root is given as the
first argument); the GPU machine and the test suite only read the committed
golden.json.

Contents:
  herm[n]      -> [x_i, w_i*exp(x_i^2)] of Internal_data/HermQuadra/herm<n>.txt (n = 1..40),
                  the Gauss-Hermite rules the reference loads in sub_quadra_hermite
                  (Source_ElVibRot/sub_Basis/sub_quadra_herm.f90:322-343);
  hh6d_levels  -> column 1 of Working_tests/MPI_tests/6D_Davidson_S0/benchmark
                  (28 Davidson levels of the 6-D Henon-Heiles SG4 L=3 model, au);
  hh21d_levels -> column 1 of Working_tests/MPI_tests/21D_Davidson_S0/benchmark
                  (22 Davidson levels of the 21-D Henon-Heiles SG4 L=2 model, au);
  pyr12d_autocorr -> Working_tests/MPI_tests/12D_propagation_S0/benchmark
                  (t in au, Re C, Im C, |C| of the 12-D pyrazine SG4 L=1 Chebyshev run);
  pyr24d_autocorr -> Working_tests/MPI_tests/24D_propagation_S0/benchmark (same columns,
                  24-D pyrazine SG4 L=2);
  pyr24d_model -> the parameters of that run's potential, read from the data statements of
                  Working_tests/MPI_tests/24D_propagation_S0/sub_system_pyrazine.f
                  (w, k1, k2 per mode, delta, lambda, in eV) and the mode rule
                  L_TO_nq_B of its shell_run (B1..B4, then B);
  wp_inputs    -> the start packets written after the namelists of two input files, in
                  the sparse form that lect_psiBasisRepnotall_nD reads
                  (Source_ElVibRot/sub_WP/sub_module_psi_io.f90:563-780):
                  Working_tests/exa_hcn-test/dat_Davidson (3 modes, 4 real packets) and
                  Working_tests/MPI_tests/12D_propagation_S0/shell_run (12 modes, one
                  complex packet on the second electronic state, ended by the file's end).
"""
import json
import os
import re
import sys

_ENTRY = re.compile(r"^\s*[-+0-9][-+0-9.eEdD\s]*$")


def packet_lines(path):
    """The packet lines (entries and 'end wp' lines) after the namelist that closes just
    before them ('/' line), up to the first other line."""
    with open(path) as f:
        lines = f.read().splitlines()

    def next_nonblank(i):
        while i < len(lines) and not lines[i].strip():
            i += 1
        return i

    start = max(i for i, ln in enumerate(lines) if ln.strip() == "/" and next_nonblank(i + 1) < len(lines)
                and _ENTRY.match(lines[next_nonblank(i + 1)]))
    out = []
    for ln in lines[start + 1:]:
        if not ln.strip():
            continue
        if ln.strip().startswith("end wp") or _ENTRY.match(ln):
            out.append(ln)
        else:
            break
    return out


def fortran_array(text, name):
    """Values of a Fortran array constructor `name(ndim) = (/ ... /)` (fixed form)."""
    m = re.search(name + r"\(ndim\)\s*=\s*\(/(.*?)/\)", text, flags=re.S)
    body = re.sub(r"\n\s*\*", " ", m.group(1)).replace("_Rkind", "")
    return [0.0 if v.strip().upper() == "ZERO" else float(v) for v in body.split(",")]


def fortran_scalar(text, name):
    return float(re.search(name + r"\s*=\s*([-0-9.eEdD+]+)_Rkind", text).group(1))


def pyrazine24_model(root):
    d = os.path.join(root, "Working_tests", "MPI_tests", "24D_propagation_S0")
    with open(os.path.join(d, "sub_system_pyrazine.f")) as f:
        src = f.read()
    with open(os.path.join(d, "shell_run")) as f:
        sh = f.read()
    b = {k: int(re.search(r"^" + k + r"=(\d+)", sh, flags=re.M).group(1)) for k in ("B1", "B2", "B3", "B4", "B")}
    with open(os.path.join(d, "run_jobs")) as f:
        L = int(f.read().split()[2])  # "./shell_run <cores> <L>"
    return dict(w=fortran_array(src, "w"), k1=fortran_array(src, "k1"), k2=fortran_array(src, "k2"),
                delta=fortran_scalar(src, "delta"), lam=fortran_scalar(src, "lambda"),
                B=[b["B1"], b["B2"], b["B3"], b["B4"]] + [b["B"]] * 20, L=L)


def main(root):
    out = {"herm": {}}
    for n in range(1, 41):
        rows = []
        with open(os.path.join(root, "Internal_data", "HermQuadra", f"herm{n}.txt")) as f:
            for line in f:
                p = line.split()
                if len(p) >= 4:
                    rows.append([float(p[1]), float(p[3])])
        out["herm"][str(n)] = rows
    with open(os.path.join(root, "Working_tests", "MPI_tests", "6D_Davidson_S0", "benchmark")) as f:
        out["hh6d_levels"] = [float(line.split()[0]) for line in f if line.strip()]
    with open(os.path.join(root, "Working_tests", "MPI_tests", "21D_Davidson_S0", "benchmark")) as f:
        out["hh21d_levels"] = [float(line.split()[0]) for line in f if line.strip()]
    with open(os.path.join(root, "Working_tests", "MPI_tests", "12D_propagation_S0", "benchmark")) as f:
        out["pyr12d_autocorr"] = [[float(v) for v in line.split()] for line in f if line.strip()]
    with open(os.path.join(root, "Working_tests", "MPI_tests", "24D_propagation_S0", "benchmark")) as f:
        out["pyr24d_autocorr"] = [[float(v) for v in line.split()] for line in f if line.strip()]
    out["pyr24d_model"] = pyrazine24_model(root)
    out["wp_inputs"] = {
        "hcn_dat_Davidson": dict(D=3, nb0=1, cplx=False, lines=packet_lines(
            os.path.join(root, "Working_tests", "exa_hcn-test", "dat_Davidson"))),
        "pyr12d_shell_run": dict(D=12, nb0=2, cplx=True, lines=packet_lines(
            os.path.join(root, "Working_tests", "MPI_tests", "12D_propagation_S0", "shell_run"))),
    }
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <root of the reference's source tree>")
    main(sys.argv[1])
