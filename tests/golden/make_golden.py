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
  pyr12d_autocorr -> Working_tests/MPI_tests/12D_propagation_S0/benchmark
                  (t in au, Re C, Im C, |C| of the 12-D pyrazine SG4 L=1 Chebyshev run).
"""
import json
import os
import sys


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
    with open(os.path.join(root, "Working_tests", "MPI_tests", "12D_propagation_S0", "benchmark")) as f:
        out["pyr12d_autocorr"] = [[float(v) for v in line.split()] for line in f if line.strip()]
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.json")
    with open(dst, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", dst)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
