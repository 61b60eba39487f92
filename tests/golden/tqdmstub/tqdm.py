"""No-op stand-in for tqdm, for importing the reference where tqdm is not
installed (the reference imports it at module level for its progress bar).
Only used behind the real package on sys.path."""


class tqdm:
    def __init__(self, iterable=None, *args, **kwargs):
        self.iterable = iterable

    def __iter__(self):
        return iter(self.iterable if self.iterable is not None else ())

    def update(self, n=1):
        pass

    def close(self):
        pass
