"""The product path has no CPU fallback: without the CUDA library every
entry point raises, and without a GPU a build raises instead of returning
anything (CPU only; the oracle is not involved)."""
import os
import subprocess
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def test_missing_library_raises():
    code = (
        "import numpy as np\n"
        "import indexing_gb300 as wah\n"
        "from indexing_gb300 import _lib\n"
        "_lib.LIB_PATH = '/nonexistent/libwah_gb300.so'\n"
        "_lib._lib = None\n"
        "for f in (lambda: wah.build_index(np.arange(10, dtype=np.uint32)),\n"
        "          lambda: wah.sort_rids_by_value(np.arange(10, dtype=np.uint32)),\n"
        "          lambda: wah.HostContext(10)):\n"
        "    try:\n"
        "        f()\n"
        "    except ImportError as e:\n"
        "        assert 'missing' in str(e)\n"
        "    else:\n"
        "        raise SystemExit('returned without the library')\n"
        "print('ok')\n")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300,
                       cwd=repo)
    assert r.returncode == 0 and r.stdout.strip().endswith("ok"), r.stdout + r.stderr


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the behaviour without a GPU")
def test_no_gpu_raises():
    import indexing_gb300 as wah
    try:
        wah._lib.load()
    except ImportError:
        pytest.skip("library not built here")
    with pytest.raises(Exception):
        wah.build_index(np.arange(1000, dtype=np.uint32))
