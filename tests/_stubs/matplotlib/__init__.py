"""Minimal import stub for matplotlib.

ProjectQ imports matplotlib at package import time (circuit drawing and
histograms).  Neither is used by the simulator path under test, and matplotlib
is not installed here, so this stub provides just the names those modules
import.  Only the test harness puts this directory on ``sys.path``.
"""


def use(*args, **kwargs):
    return None


pyplot = None
