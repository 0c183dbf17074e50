"""include/gb300mps.h is plain C: a C99 program using the documented calls
compiles with -Wall -Werror, links against libgb300mps.so and, without a
GPU, reports the missing device through the status codes."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r"""
#include <stdio.h>
#include "gb300mps.h"

int main(void) {
  mps_cfg cfg = {0, 0};
  mps_ctx* ctx = NULL;
  mps_prog* p = NULL;
  int q01[2] = {0, 1};
  double z[2];
  int rc = mps_ctx_create(&cfg, &ctx);
  if (rc != MPS_OK) {
    printf("no context: %d %s\n", rc, mps_last_error());
    return 2;
  }
  if (mps_program_begin(ctx, 12, 64, 1e-14, MPS_TRUNC_EXATN, MPS_PREC_FP64, 0, &p) != MPS_OK ||
      mps_gate_named(p, "H", q01, 1, NULL, 0) != MPS_OK || mps_gate_named(p, "CNOT", q01, 2, NULL, 0) != MPS_OK ||
      mps_submit(p) != MPS_OK || mps_expect_pauli(p, "ZZIIIIIIIIII", 1, NULL, z) != MPS_OK) {
    printf("error: %s\n", mps_last_error());
    return 1;
  }
  printf("zz %.12f\n", z[0]);
  mps_program_destroy(p);
  mps_ctx_destroy(ctx);
  return 0;
}
"""


def test_header_is_c99_and_the_library_links(tmp_path):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    from tnqvm_gb300 import build as B
    lib = B.build()
    src = tmp_path / "example.c"
    src.write_text(PROGRAM)
    exe = str(tmp_path / "example")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", exe, "-L", os.path.dirname(lib), "-lgb300mps", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    import torch
    if torch.cuda.is_available():
        assert r.returncode == 0 and abs(float(r.stdout.split()[1]) - 1.0) < 1e-10, r.stdout
    else:
        assert r.returncode == 2 and "no context: 5" in r.stdout, r.stdout
