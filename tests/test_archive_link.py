"""The static archive the R package links (`python -m vectra_gb300.build
--archive`): a C host that calls the four node constructors and defines
its own vectra_error (as the engine's src/error.c does) links against
libvgpu.a with the libraries the integration notes list, and its own
vectra_error takes precedence over libvgpu's weak default.  Link only: the
program is not run (no device is needed for this check)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

HOST = r"""
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include "vgpu.h"

int engine_error_calls = 0;
void vectra_error(const char *fmt, ...) {   /* the engine's own definition */
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
    engine_error_calls++;
    exit(3);
}

int main(int argc, char **argv) {
    (void)argv;
    if (argc > 5) {   /* never taken: the calls only have to link */
        filter_node_create(NULL, NULL);
        project_node_create(NULL, 0, NULL);
        group_agg_node_create(NULL, 0, NULL, 0, NULL, NULL);
        join_node_create(NULL, NULL, JOIN_INNER, 0, NULL, NULL, NULL);
    }
    return engine_error_calls;
}
"""


def test_r_package_link_line(tmp_path):
    from vectra_gb300 import build
    build.build(archive=True)
    archive = os.path.join(ROOT, "vectra_gb300", "libvgpu.a")
    assert os.path.exists(archive)
    cuda = os.path.dirname(build._cuda_include())
    src = tmp_path / "host.c"
    src.write_text(HOST)
    exe = tmp_path / "host"
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("no gcc")
    subprocess.run([gcc, "-std=gnu11", "-c", str(src), "-o", str(tmp_path / "host.o"),
                    "-I", os.path.join(ROOT, "include"), "-I", build._cuda_include()], check=True)
    r = subprocess.run(["g++", "-o", str(exe), str(tmp_path / "host.o"), archive,
                        "-L" + os.path.join(cuda, "lib64"), "-lcudart_static", "-lnvrtc", "-ldl", "-lrt",
                        "-lpthread", "-lstdc++"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    nm = subprocess.run(["nm", str(exe)], capture_output=True, text=True, check=True).stdout
    # the host's strong vectra_error is the one linked (a weak one would show as W)
    lines = [l for l in nm.splitlines() if l.endswith(" vectra_error")]
    assert lines and all(" T " in l for l in lines), lines
