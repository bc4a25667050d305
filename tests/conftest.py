"""Test configuration: registers the ``gpu`` marker and makes sure the in-tree
libraries exist (the product .so and the oracle .so) before tests import them.
GPU tests do not skip when CUDA is missing: they fail, so a GPU run can never
pass without the kernels."""
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    import importlib.util

    # by path: importing the package would load the library before it is built
    spec = importlib.util.spec_from_file_location("mitrace_gb300_build", ROOT / "mitrace_gb300" / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    b.build_product()
    b.build_oracle()
