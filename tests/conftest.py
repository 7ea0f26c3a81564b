import os
import sys

# The autotuner's choices change the order of some sums (the split count of X G^T, the CP-ALS
# chunk rows).  Tests keep them in memory only, so results never depend on a tuning cache left
# on the machine by an earlier process.
os.environ["FH_TUNE_CACHE"] = ""

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (ROOT, os.path.join(ROOT, "fast-higashi_gb300"), os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built extension")
