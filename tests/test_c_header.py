"""The drop-in boundary is a C ABI: a C99 program (no C++) includes
include/pakman_gb300.h with every warning an error, links libpakman_gb300.so, calls it,
and sees the struct layouts the Python mirror uses.  Without a GPU the context call
fails with PK_ERR_NO_DEVICE (there is no CPU fallback); with one it succeeds."""
import ctypes
import os
import shutil
import subprocess

import pytest

from pakman_plus_gb300 import build as pkbuild
from pakman_plus_gb300 import capi

PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "pakman_gb300.h"

int main(void) {
  pk_params p;
  pk_params_default(&p);
  if (p.k != 32 || p.num_buckets != 21) return 2;
  if (strcmp(pk_status_string(PK_ERR_EMPTY), pk_status_string(PK_OK)) == 0) return 3;
  pk_server_config cfg;
  pk_server_config_default(&cfg, 8);
  if (cfg.small_sms != 0 || cfg.reserved_small != 1) return 4;
  printf("%zu %zu %zu %zu %zu %zu\n", sizeof(pk_params), sizeof(pk_summary), sizeof(pk_request),
         sizeof(pk_request_info), sizeof(pk_server_config), sizeof(pk_batch_set));
  pk_ctx* ctx = NULL;
  pk_status st = pk_ctx_create(0, 0, &ctx);
  printf("%d\n", (int)st);
  if (st == PK_OK) pk_ctx_destroy(ctx);
  return (st == PK_OK || st == PK_ERR_NO_DEVICE) ? 0 : 5;
}
"""


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_header_compiles_as_c99_and_links(tmp_path):
    pkbuild.build()
    src = tmp_path / "use_pk.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "use_pk"
    lib_dir = os.path.dirname(pkbuild.LIB)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", "-I", pkbuild.INCLUDE,
                    str(src), "-o", str(exe), f"-L{lib_dir}", "-lpakman_gb300", f"-Wl,-rpath,{lib_dir}"],
                   check=True, capture_output=True, text=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, (r.returncode, r.stdout, r.stderr)
    sizes, status = r.stdout.split("\n")[:2]
    assert [int(x) for x in sizes.split()] == [
        ctypes.sizeof(capi.PkParams), ctypes.sizeof(capi.PkSummary), ctypes.sizeof(capi.PkRequest),
        ctypes.sizeof(capi.PkRequestInfo), ctypes.sizeof(capi.PkServerConfig), ctypes.sizeof(capi.PkBatchSet)]
    assert int(status) in (capi.PK_OK, capi.PK_ERR_NO_DEVICE)
