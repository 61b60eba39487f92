"""No-op pyplot stand-in: every attribute is a callable that returns None."""


def __getattr__(name):
    def _noop(*args, **kwargs):
        return None

    return _noop
