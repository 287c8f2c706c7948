"""The boundary is a plain C ABI: include/tn_mps.h compiles as strict C99
(-pedantic -Werror) and a C host (tests/c_host/trajectory.c) links against
libtnmps and runs a seeded trajectory through it.  Without a GPU the
library refuses loudly (exit 3, "no CUDA device"); with one, the C host's
per-layer entropies equal the Python mirror's bit for bit."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]


def _build(pkg, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = pkg.library_path().parent
    exe = tmp_path / "trajectory"
    r = subprocess.run([cc, "-std=c99", "-Wall", "-Wextra", "-Werror", "-pedantic", f"-I{ROOT / 'include'}",
                        str(ROOT / "tests" / "c_host" / "trajectory.c"), f"-L{libdir}", "-ltnmps",
                        f"-Wl,-rpath,{libdir}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_host_compiles_and_refuses_without_a_device(pkg, tmp_path):
    exe = _build(pkg, tmp_path)
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present (the run is covered by the GPU test)")
    r = subprocess.run([str(exe), "8", "3", "0.2", "16", "5"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 3 and "no CUDA device" in r.stdout


@pytest.mark.gpu
def test_c_host_matches_the_python_mirror(pkg, tmp_path):
    exe = _build(pkg, tmp_path)
    n, depth, p, chi, seed = 10, 8, 0.2, 16, 5
    r = subprocess.run([str(exe), str(n), str(depth), str(p), str(chi), str(seed)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stderr
    ents = [float(line.split()[3]) for line in r.stdout.splitlines() if line.startswith("layer")]
    m = pkg.MPS.new_qubits(n, pkg.Trunc.both(chi, 1e-12), "f64")
    want = []
    for t in range(depth):
        m.apply_bilayer(*pkg.gen_layer(seed, 0, t, n, p))
        want.append(m.entropy_vn(n // 2 - 1))
    assert ents == want
