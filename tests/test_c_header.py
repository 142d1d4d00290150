"""include/ati.h from plain C (CPU, no device): a C99 program compiled with
-std=c99 -pedantic -Wall -Werror against the header and linked with the
built library calls the host-only entry points.  It reads an ati_config_t
that the Python binding wrote as raw bytes (so the C layout and the ctypes
mirror must agree), builds the dense zeta operator of one block, and checks
two refusals; the operator it prints must equal the Python binding's."""
import ctypes
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "ati.h"

int main(int argc, char **argv) {
  ati_config_t cfg;
  if (argc < 2) return 9;
  FILE *f = fopen(argv[1], "rb");
  if (!f || fread(&cfg, sizeof cfg, 1, f) != 1) return 10;
  fclose(f);
  if (ati_abi_version() != ATI_ABI_VERSION) return 11;
  static double m[64 * 64];
  int32_t n = 0;
  if (ati_dense_zeta_operator(&cfg, 1, m, &n) != ATI_OK) return 12;
  ati_config_t bad = cfg;
  bad.bkx = 2;
  ati_handle_t *h = NULL;
  if (ati_create(&bad, &h) != ATI_EINVAL || h != NULL || strlen(ati_last_error(NULL)) == 0) return 13;
  if (ati_deriv_lines_noalloc(m, m, 1, 5000, NULL) != ATI_EINVAL) return 14;
  printf("%d\n", (int)n);
  for (int i = 0; i < n * n; i++) printf("%.17g\n", m[i]);
  return 0;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_from_c99(ati_lib, tmp_path):
    from tandemproject_gb300.config import small_case
    from tandemproject_gb300.solver import dense_zeta_operator
    cfg = small_case(lzebk=(19,))
    (tmp_path / "cfg.bin").write_bytes(bytes(cfg.to_c()))
    src = tmp_path / "use_ati.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "use_ati"
    libdir = os.path.dirname(ati_lib)
    subprocess.run(["gcc", "-std=c99", "-pedantic", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-o", str(exe), "-L", libdir, "-lati", "-Wl,-rpath," + libdir], check=True)
    r = subprocess.run([str(exe), str(tmp_path / "cfg.bin")], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    vals = r.stdout.split()
    n = int(vals[0])
    m = np.array([float(v) for v in vals[1:]]).reshape(n, n)
    assert n == 20 and np.array_equal(m, dense_zeta_operator(cfg, 1))
    assert ctypes.sizeof(type(cfg.to_c())) == len((tmp_path / "cfg.bin").read_bytes())
