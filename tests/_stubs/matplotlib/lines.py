"""Import stub for matplotlib.lines."""


class Line2D:
    pass
