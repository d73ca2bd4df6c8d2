"""Stand-in for hydra: ``main`` is an identity decorator."""


def main(*args, **kwargs):
    def deco(fn):
        return fn
    return deco


def compose(*a, **k):
    raise NotImplementedError


def initialize(*a, **k):
    raise NotImplementedError


def initialize_config_dir(*a, **k):
    raise NotImplementedError
