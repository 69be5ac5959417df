"""Import stub for matplotlib.collections."""


class LineCollection:
    pass


class PatchCollection:
    pass
