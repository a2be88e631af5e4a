"""The checked build (libvoxtrees_cuda_checked.so, -DVOX_CUDA_CHECKED): every
search load -- tree records, leaf voxels, light-tree nodes and spheres --
first checks its index against the uploaded arrays and ends the search with
VOX_CUDA_ERANGE instead of reading outside them.  It stands in for a memory
checker on the search kernels: the GPU parity suites, run against it in a
child process, must pass unchanged -- no index outside the arrays on any valid
tree, and every result still the oracle's.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SUITES = ["tests/test_gpu_parity.py", "tests/test_gpu_lights.py", "tests/test_gpu_custom_camera.py",
          "tests/test_gpu_render_best.py", "tests/test_gpu_batch.py", "tests/test_gpu_tree_edit.py"]


@pytest.fixture(scope="module")
def checked_lib():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from voxvision_gb300.build import build
    build()
    return build(checked=True)


def _child(lib, args, timeout):
    env = dict(os.environ, VOXTREES_CUDA_LIB=lib)
    return subprocess.run([sys.executable, *args], env=env, cwd=ROOT, capture_output=True, text=True,
                          timeout=timeout)


def test_builds_report_which_they_are(checked_lib):
    r = _child(checked_lib, ["-c", "import voxvision_gb300 as v; print(v.lib().vox_cuda_build_checked())"], 300)
    assert r.returncode == 0 and r.stdout.strip() == "1", r.stderr[-2000:]
    if not os.environ.get("VOXTREES_CUDA_LIB"):
        import voxvision_gb300 as vg
        assert vg.lib().vox_cuda_build_checked() == 0
    import voxvision_gb300 as vg
    assert "checked build" in vg.lib().vox_cuda_strerror(-12).decode()


def test_parity_suites_pass_on_the_checked_build(checked_lib):
    r = _child(checked_lib, ["-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider", *SUITES], 1800)
    assert r.returncode == 0, (r.stdout[-4000:], r.stderr[-2000:])
    summary = r.stdout.strip().splitlines()[-1]
    print("checked build:", summary)
    assert " passed" in summary and "skipped" not in summary and "deselected" not in summary, summary
    assert int(summary.split()[0]) >= 40, summary
