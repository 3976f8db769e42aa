import importlib
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# the package directory is "ace-tn_gb300"; expose it as acetn_gb300
sys.modules.setdefault("acetn_gb300", importlib.import_module("ace-tn_gb300"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")
