"""Minimal stand-in for PyYAML: the reference only loads optional user config
files (shenfun/config.py:96-116), which do not exist in this setup."""


def load(stream, Loader=None):
    return {}


safe_load = load


def dump(data, stream=None, **kw):
    if stream is not None:
        stream.write(repr(data))
    return repr(data)


class FullLoader:  # noqa: D401 - placeholder
    pass


Loader = SafeLoader = FullLoader
