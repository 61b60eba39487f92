"""Stand-in for matplotlib.colors: only the LogNorm name is needed at import time."""


class LogNorm:
    def __init__(self, *args, **kwargs):
        pass
