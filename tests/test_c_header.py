"""include/evr_gpu.h is a plain C ABI: it compiles as strict C99, and a C program links
against libevrgpu.so and runs its host-only entry points (context on the host, table
sizes, wave-packet file round trip) without a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "evr_gpu.h"

int main(int argc, char **argv) {
  if (argc < 2) return 9;
  int Aq[3] = {1, 1, 1}, Bq[3] = {2, 2, 2};
  int idx[4] = {0, 0, -1, -1};
  double coef[1] = {0.5};
  evr_problem_desc d;
  memset(&d, 0, sizeof d);
  d.kind = EVR_BASIS_SG4; d.D = 3; d.nb0 = 1; d.LG = 2; d.LB = 2;
  d.Aq = Aq; d.Bq = Bq; d.Ab = Aq; d.Bb = Bq;
  d.n_mono = 1; d.mono_coef = coef; d.mono_idx = idx; d.keo_type = 1;
  evr_ctx *ctx = NULL;
  int rc = evr_create(&ctx, &d, -1);
  if (rc != EVR_OK) { printf("create %d %s\n", rc, evr_last_error(ctx)); return 1; }
  evr_sizes_t s;
  if (evr_sizes(ctx, &s) != EVR_OK || s.N < 1) return 2;
  double psi[4096], back[4096];
  int n = 0; int64_t dropped = -1;
  if (s.N > 4096) return 3;
  for (int64_t k = 0; k < s.N; ++k) psi[k] = 0.25 * (double)(k % 7) - 0.5;
  if (evr_psi_write(ctx, argv[1], EVR_WP_FORMATTED_V1, psi, s.N, 1, 0, 0.0) != EVR_OK) return 4;
  if (evr_psi_read(ctx, argv[1], back, s.N, 1, 0, &n, &dropped) != EVR_OK || n != 1 || dropped != 0) return 5;
  for (int64_t k = 0; k < s.N; ++k) if (back[k] != psi[k]) return 6;
  if (evr_hpsi_host(ctx, psi, s.N, back, s.N, 1, EVR_LAYOUT_COLMAJOR, EVR_PREC_FP64) != EVR_EDEVICE) return 7;
  printf("ok N=%lld terms=%lld\n", (long long)s.N, (long long)s.n_terms);
  evr_destroy(ctx);
  return 0;
}
"""


def test_header_is_strict_c99_and_links(tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    from evrgpu import lib as E

    so = E.load()._name
    src = tmp_path / "prog.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "prog"
    cmd = ["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
           str(src), so, "-Wl,-rpath," + os.path.dirname(so), "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path / "wp")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.startswith("ok"), (r.returncode, r.stdout, r.stderr)
