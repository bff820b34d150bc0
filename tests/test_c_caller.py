"""The C ABI from a plain C99 caller, as the reference would link it (no GPU).

A small C program is compiled with gcc against include/sdmd_gpu.h and
include/sdmd_host.h and linked with the two libraries.  It runs the calls that
need no device: the ABI version and error strings, the glibc-compatible rand()
helpers (against the C library's own srand/rand in the same process), reading
parameter.txt, and building the reference's initial state from a .gro through
sdmd_host.h.  The device count is queried; without a GPU it reports none.
"""
import os
import shutil
import subprocess

import numpy as np

from sdmd_gb300 import build

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SRC = r"""
#include <stdio.h>
#include <stdlib.h>
#include "sdmd_gpu.h"
#include "sdmd_host.h"

int main(int argc, char **argv) {
    printf("abi %d\n", sdmd_gpu_abi_version());
    printf("strerror %s\n", sdmd_gpu_strerror(SDMD_ECAPACITY) ? "ok" : "null");
    sdmd_rng r;
    sdmd_rng_seed(&r, 1575263273u);
    srand(1575263273u);
    int same = 1;
    for (int k = 0; k < 2000; k++) same &= sdmd_rng_next(&r) == rand();
    printf("rng %s\n", same ? "ok" : "differs");
    sdmd_params p;
    char path[4096];
    snprintf(path, sizeof path, "%s/parameter.txt", argv[1]);
    if (sdmd_read_parameters(path, &p) != SDMD_OK) { printf("parameters failed\n"); return 1; }
    sdmd_host_system *h = NULL;
    char err[512];
    int rc = sdmd_build_system(argv[1], "sys.gro", &p, NULL, 1575263273u, 20000, &h, err, sizeof err);
    if (rc != SDMD_OK) { printf("build failed: %s\n", err); return 1; }
    const sdmd_system *s = sdmd_host_view(h);
    printf("atoms %d x1 %a\n", s->n_atoms, s->x[1]);
    snprintf(path, sizeof path, "%s/out_trj.gro", argv[1]);
    rc = sdmd_write_gro(path, 0, s, sdmd_host_atom_names(h), sdmd_host_residue_names(h));
    printf("gro %d\n", rc);
    sdmd_host_free(h);
    int32_t n = -1;
    rc = sdmd_gpu_device_count(&n);
    printf("devices rc %d n %d\n", rc, n);
    return 0;
}
"""


def test_plain_c_caller(golden, tmp_path):
    gpu = build.build_gpu()
    host = build.build_host()
    d = golden("ala10_nvt")
    data = tmp_path / "data"
    data.mkdir()
    shutil.copytree(os.path.join(REPO, "sdmd_gb300", "data", "Library_Ding"), data / "Library_Ding")
    (data / "parameter.txt").write_bytes(bytes(d["meta/parameter"]))
    (data / "sys.gro").write_bytes(bytes(d["meta/gro"]))
    src = tmp_path / "caller.c"
    src.write_text(SRC)
    exe = tmp_path / "caller"
    libdir = os.path.dirname(gpu)
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(REPO, "include"), str(src), "-o", str(exe),
                    "-L", libdir, "-lsdmd_gpu", "-lsdmd_host", f"-Wl,-rpath,{libdir}"], check=True)
    assert os.path.dirname(host) == libdir
    out = subprocess.run([str(exe), str(data)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    lines = dict(l.split(" ", 1) for l in out.stdout.splitlines())
    assert lines["strerror"] == "ok" and lines["rng"] == "ok"
    atoms, x1 = lines["atoms"].split(" x1 ")
    assert int(atoms) == 59
    assert float.fromhex(x1) == float(d["pre/x"][1])   # the reference's initial state
    assert lines["gro"] == "0"                            # the trajectory writer, from C
    gro = (data / "out_trj.gro").read_text().splitlines()
    assert gro[0] == "model" and int(gro[1]) == 59 and len(gro) == 62 and gro[2][10:15].strip() == "N"
