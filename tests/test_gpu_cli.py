"""The reference's command line on the GPU: `./ALG file.mtx source iters`
(main.cu:18-159) for every binary name, its `processing : ... MTEPS,` and
`validation : PASS` lines, and the binary CSR cache as input."""
import os
import re
import subprocess
import tempfile

import pytest

import multigraph_gb300 as mg

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
MTX = os.path.join(ROOT, "tests", "golden", "mtx")
LINE = re.compile(r"processing : ([0-9.]+) ms,([0-9.]+) MTEPS,\s*validation : PASS")


def _run(name, path, source, iters=2, env=None):
    r = subprocess.run([os.path.join(mg.BIN_DIR, name), path, str(source), str(iters)], capture_output=True,
                       text=True, timeout=300, env=dict(os.environ, **(env or {})))
    assert r.returncode == 0, (name, path, r.stdout, r.stderr)
    m = LINE.search(r.stdout)
    assert m, (name, path, r.stdout)
    return float(m.group(1)), float(m.group(2))


@pytest.mark.parametrize("name", ["BFS", "SSSP", "BC", "CC", "DATA_DRIVEN_PR", "TOPOLOGY_DRIVEN_PR"])
@pytest.mark.parametrize("fixture", ["rmat8.mtx", "lattice6x7.mtx", "twocomp.mtx", "renumber.mtx"])
def test_cli_validates(name, fixture):
    _run(name, os.path.join(MTX, fixture), 1)


def test_cli_generated_rmat_and_binary_cache():
    tmp = tempfile.mkdtemp()
    h = mg.HostGraph.rmat(12, 16, seed=7)
    p = os.path.join(tmp, "r12.mtx")
    h.write_mtx(p, True)
    cache = os.path.join(tmp, "r12.mgcsr")
    _run("SSSP", p, 1, env={"MG_CSR_SAVE": cache})
    assert os.path.getsize(cache) > 0
    back = mg.HostGraph.load_csr(cache)
    assert back.nv == h.nv and back.ne == h.ne
    for name in ("BFS", "SSSP", "BC", "CC"):
        _run(name, cache, 0)
