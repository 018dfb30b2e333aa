import os
import sys

ROOT = os.path.abspath(os.path.join(os.path.dirname(__file__), ".."))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs an sm_103 GPU (runs the CUDA path)")
    config.addinivalue_line("markers", "reference: needs the reference sources on this machine")
