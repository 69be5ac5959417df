"""Minimal import stub for networkx (imported by ProjectQ's 2-D grid mapper at
package import time; not used by the simulator tests, absent on the GPU host)."""


class Graph:
    def __init__(self, *args, **kwargs):
        raise RuntimeError("networkx is not available in the test environment")
