"""The C ABI from plain C (gcc, -std=c99 -Wall -Werror): both headers compile
as C, and programs link against the two libraries.  The host library runs
end to end (generate a flow instance with every node row, remove its
dependent rows, read the counts); the GPU library is linked and its one
entry point that touches no device (help_pcg_default_options) is called."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "help_gb300", "_lib")
INC = os.path.join(ROOT, "include")

LP_PROGRAM = r"""
#include <stdio.h>
#include <string.h>
#include "help_lp.h"

int main(void) {
    help_lp_spec spec;
    memset(&spec, 0, sizeof spec);
    spec.kind = HELP_LP_MCF;
    spec.grid = 6;
    spec.commodities = 3;
    spec.pairs_per_commodity = 2;
    spec.mcf_ungrounded = 1;
    help_lp lp, reduced;
    if (help_lp_generate(&spec, 5, &lp) != 0) return 1;
    int32_t removed[4096];
    if (lp.m > 4096) return 2;
    int rc = help_lp_remove_dependent_rows(&lp, 1e-8, &reduced, removed);
    printf("%d %d %d\n", lp.m, rc, reduced.m);
    help_lp_free(&reduced);
    help_lp_free(&lp);
    return rc < 0 ? 3 : 0;
}
"""

GPU_PROGRAM = r"""
#include <stdio.h>
#include "help_gpu.h"
#include "help_lp.h"

int main(void) {
    help_pcg_options opt;
    help_pcg_default_options(&opt);
    help_ne_backend be = {0};
    printf("%d %d\n", opt.pivots > 0, be.matvec == 0);
    return 0;
}
"""


def build_and_run(tmp_path, name, source, lib, run=True):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    src = tmp_path / (name + ".c")
    exe = tmp_path / name
    src.write_text(source)
    cmd = [gcc, "-std=c99", "-Wall", "-Werror", "-I", INC, str(src), "-L", LIB, "-l" + lib,
           "-Wl,-rpath," + LIB, "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    if not run:
        return None
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout.split()


def test_host_library_from_c(tmp_path):
    m, rc, m_reduced = map(int, build_and_run(tmp_path, "lp_c", LP_PROGRAM, "help_lp"))
    # 6 x 6 grid, 3 commodities, every node row: 3 x 36 node rows + 120 arc rows
    assert m == 3 * 36 + 120
    assert rc == 3 and m_reduced == m - 3


def test_gpu_library_links_from_c(tmp_path):
    if not os.path.exists(os.path.join(LIB, "libhelp_gpu.so")):
        pytest.skip("GPU library not built")
    cudart = [p for p in ("/usr/local/cuda/lib64", "/usr/local/cuda/targets/%s-linux/lib" % os.uname().machine)
              if os.path.isdir(p)]
    env_paths = ":".join(cudart + [os.environ.get("LD_LIBRARY_PATH", "")])
    out = build_and_run(tmp_path, "gpu_c", GPU_PROGRAM, "help_gpu", run=False)
    assert out is None
    r = subprocess.run([str(tmp_path / "gpu_c")], capture_output=True, text=True, timeout=120,
                       env=dict(os.environ, LD_LIBRARY_PATH=env_paths))
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.split() == ["1", "1"]
