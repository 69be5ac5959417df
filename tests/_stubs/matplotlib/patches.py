"""Import stub for matplotlib.patches."""


class Arc:
    pass


class Circle:
    pass


class Rectangle:
    pass
