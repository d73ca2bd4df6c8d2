"""Stand-in for the parts of omegaconf that the reference's src/class uses.

DictConfig: a dict with attribute access; ListConfig: a list; OmegaConf.create
converts nested dicts/lists.  Used only to run the reference for fixtures.
"""
from .listconfig import ListConfig


class DictConfig(dict):
    def __getattr__(self, k):
        try:
            return self[k]
        except KeyError as e:
            raise AttributeError(k) from e

    def __setattr__(self, k, v):
        self[k] = v

    def copy(self):
        return OmegaConf.create(_plain(self))


def _plain(x):
    if isinstance(x, dict):
        return {k: _plain(v) for k, v in x.items()}
    if isinstance(x, list):
        return [_plain(v) for v in x]
    return x


def _wrap(x):
    if isinstance(x, DictConfig):
        return x
    if isinstance(x, dict):
        return DictConfig({k: _wrap(v) for k, v in x.items()})
    if isinstance(x, ListConfig):
        return x
    if isinstance(x, (list, tuple)):
        return ListConfig([_wrap(v) for v in x])
    return x


class OmegaConf:
    @staticmethod
    def create(obj=None):
        return _wrap(_plain(obj if obj is not None else {}))

    @staticmethod
    def to_container(cfg, resolve=True):
        return _plain(cfg)
