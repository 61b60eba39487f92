"""Stand-in for matplotlib.patches (imported, never used by the golden generator)."""


def __getattr__(name):
    def _noop(*args, **kwargs):
        return None

    return _noop
