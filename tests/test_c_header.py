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


DENSITY_PROGRAM = r"""
#include <stdio.h>
#include "gb300mps.h"

int main(void) {
  mps_cfg cfg = {0, 0};
  mps_ctx* ctx = NULL;
  mps_prog* rho = NULL;
  const double a = 0.99498743710662, b = 0.05773502691896258; /* depolarizing, p = 0.01 */
  const double kraus[4 * 8] = {a, 0, 0, 0, 0, 0, a, 0,  0, 0, b, 0, b, 0, 0, 0,
                               0, 0, 0, -b, 0, b, 0, 0, b, 0, 0, 0, 0, 0, -b, 0};
  int q0 = 0;
  double dm[2 * 4];
  int rc = mps_ctx_create(&cfg, &ctx);
  if (rc != MPS_OK) {
    printf("no context: %d %s\n", rc, mps_last_error());
    return 2;
  }
  if (mps_program_begin(ctx, 3, 64, -1.0, MPS_TRUNC_EXATN, MPS_PREC_FP64, MPS_FLAG_DENSITY, &rho) != MPS_OK ||
      mps_gate_named(rho, "X", &q0, 1, NULL, 0) != MPS_OK || mps_channel1(rho, 0, 4, kraus) != MPS_OK ||
      mps_density_matrix(rho, 1, &q0, dm) != MPS_OK) {
    printf("error: %s\n", mps_last_error());
    return 1;
  }
  printf("rho00 %.12f rho11 %.12f\n", dm[0], dm[6]);
  mps_program_destroy(rho);
  mps_ctx_destroy(ctx);
  return 0;
}
"""


def test_density_example_is_c99(tmp_path):
    """The noisy-circuit example of the C-library documentation compiles as
    C99 with -Werror and links; with a GPU it gives the reference test's
    depolarized density matrix diag(0.00666667, 0.99333333)."""
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("gcc not available")
    from tnqvm_gb300 import build as B
    lib = B.build()
    src = tmp_path / "density.c"
    src.write_text(DENSITY_PROGRAM)
    exe = str(tmp_path / "density")
    subprocess.run([gcc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", exe, "-L", os.path.dirname(lib), "-lgb300mps", "-Wl,-rpath," + os.path.dirname(lib)],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    import torch
    if torch.cuda.is_available():
        f = r.stdout.split()
        assert r.returncode == 0 and abs(float(f[1]) - 0.02 / 3) < 1e-12 and abs(float(f[3]) - (1 - 0.02 / 3)) < 1e-12
    else:
        assert r.returncode == 2 and "no context: 5" in r.stdout, r.stdout
