"""Configuration surface of the reference's simulation driver, without Hydra.

The reference composes ``conf/config_fp.yaml`` with Hydra/OmegaConf
(conf/config_fp.yaml:1-11) and expands list-valued fields into runs with
``initialize_runs`` (src/class/engine.py:13-38).  Neither Hydra nor OmegaConf
is needed here: ``compose`` reads the same YAML files with a small loader for
the subset they use, applies ``group.key=value`` / ``+key=value`` overrides,
and returns nested plain dicts (an OmegaConf ``DictConfig`` is accepted
anywhere a dict is).
"""
from __future__ import annotations

import copy
import os
import re
from typing import Any, Dict, List, Optional

# OmegaConf's YAML loader also reads exponent-only numbers such as ``1e12`` as
# floats (plain YAML 1.1 would read them as strings); the reference relies on it.
_INT = re.compile(r"^[-+]?[0-9][0-9_]*$")
_FLOAT = re.compile(
    r"^[-+]?(?:[0-9][0-9_]*\.[0-9_]*(?:[eE][-+]?[0-9]+)?|\.[0-9_]+(?:[eE][-+]?[0-9]+)?"
    r"|[0-9][0-9_]*[eE][-+]?[0-9]+|\.inf|\.nan)$", re.IGNORECASE)


def parse_scalar(text: str) -> Any:
    s = text.strip()
    if s == "" or s in ("~", "null", "Null", "NULL"):
        return None
    if s in ("true", "True", "TRUE"):
        return True
    if s in ("false", "False", "FALSE"):
        return False
    if (s[0] == s[-1]) and s[0] in "'\"" and len(s) >= 2:
        return s[1:-1]
    if s.startswith("[") and s.endswith("]"):
        inner = s[1:-1].strip()
        return [] if not inner else [parse_scalar(p) for p in _split_flow(inner)]
    if _INT.match(s):
        return int(s.replace("_", ""))
    if _FLOAT.match(s):
        low = s.lower()
        if low.endswith(".inf"):
            return float("-inf") if low.startswith("-") else float("inf")
        if low.endswith(".nan"):
            return float("nan")
        return float(s.replace("_", ""))
    return s


def _split_flow(s: str) -> List[str]:
    out, depth, cur = [], 0, ""
    for ch in s:
        if ch == "," and depth == 0:
            out.append(cur)
            cur = ""
            continue
        depth += ch == "["
        depth -= ch == "]"
        cur += ch
    out.append(cur)
    return out


def _strip_comment(line: str) -> str:
    quote = None
    for i, ch in enumerate(line):
        if quote:
            if ch == quote:
                quote = None
        elif ch in "'\"":
            quote = ch
        elif ch == "#" and (i == 0 or line[i - 1] in " \t"):
            return line[:i]
    return line


def _read_group_file(path: str) -> Dict[str, Any]:
    """Read a YAML file whose top level may contain ``- item`` lists."""
    with open(path, "r", encoding="utf-8") as f:
        raw = [_strip_comment(l).rstrip() for l in f.read().splitlines()]
    raw = [l for l in raw if l.strip()]
    # Rewrite "key:\n  - a\n  - b" into "key: [a, b]" before the mapping parse.
    out: List[str] = []
    i = 0
    while i < len(raw):
        line = raw[i]
        body = line.strip()
        if body.endswith(":") and i + 1 < len(raw) and raw[i + 1].strip().startswith("- "):
            items = []
            j = i + 1
            while j < len(raw) and raw[j].strip().startswith("- "):
                items.append(raw[j].strip()[2:].strip())
                j += 1
            out.append(f"{line} [{', '.join(items)}]")
            i = j
            continue
        out.append(line)
        i += 1
    tmp = "\n".join(out)
    return _parse_mapping(tmp, path)


def _parse_mapping(text: str, path: str) -> Dict[str, Any]:
    root: Dict[str, Any] = {}
    stack = [(-1, root)]
    for line in text.splitlines():
        indent = len(line) - len(line.lstrip(" "))
        body = line.strip()
        while len(stack) > 1 and indent <= stack[-1][0]:
            stack.pop()
        parent = stack[-1][1]
        if ":" not in body:
            raise ValueError(f"unsupported YAML line in {path}: {line!r}")
        key, _, val = body.partition(":")
        key = key.strip()
        if val.strip() == "":
            child: Dict[str, Any] = {}
            parent[key] = child
            stack.append((indent, child))
        else:
            parent[key] = parse_scalar(val)
    return root


def read_yaml(path: str) -> Dict[str, Any]:
    """Public YAML reader for the reference's ``conf/`` files."""
    return _read_group_file(path)


def _set_path(cfg: Dict[str, Any], dotted: str, value: Any, add: bool) -> None:
    parts = dotted.split(".")
    node = cfg
    for p in parts[:-1]:
        if p not in node or not isinstance(node[p], dict):
            if not add:
                raise KeyError(f"override of unknown key '{dotted}' (use +{dotted}=...)")
            node[p] = {}
        node = node[p]
    if parts[-1] not in node and not add:
        raise KeyError(f"override of unknown key '{dotted}' (use +{dotted}=...)")
    node[parts[-1]] = value


def compose(conf_dir: str, overrides: Optional[List[str]] = None,
            config_name: str = "config_fp") -> Dict[str, Any]:
    """Compose ``config_name`` with its default groups and apply overrides.

    Mirrors what ``@hydra.main(config_path=CONFIG_DIR, config_name="config_fp")``
    hands to ``simulate`` (src/class/simulate.py:11): the primary file's own keys
    plus one file per config group named in ``defaults``.  Overrides use Hydra's
    syntax: ``group=option`` picks a group file, ``group.key=value`` replaces a
    value, ``+key=value`` adds a new key.
    """
    overrides = list(overrides or [])
    primary = read_yaml(os.path.join(conf_dir, f"{config_name}.yaml"))
    defaults = primary.pop("defaults", [])
    groups: Dict[str, str] = {}
    for d in defaults:
        if isinstance(d, dict):
            for k, v in d.items():
                groups[k] = v
        elif isinstance(d, str) and ":" in d:
            k, v = d.split(":", 1)
            groups[k.strip()] = parse_scalar(v)
    value_ovr = []
    for o in overrides:
        key, _, val = o.partition("=")
        k = key.lstrip("+")
        if k in groups and "." not in k and not key.startswith("+"):
            groups[k] = val
        else:
            value_ovr.append((key, val))
    cfg: Dict[str, Any] = {}
    for k, v in primary.items():
        if k != "hydra":
            cfg[k] = copy.deepcopy(v)
    for g, opt in groups.items():
        cfg[g] = read_yaml(os.path.join(conf_dir, g, f"{opt}.yaml"))
    for key, val in value_ovr:
        _set_path(cfg, key.lstrip("+"), parse_scalar(val), add=key.startswith("+"))
    return cfg


def _is_list(v: Any) -> bool:
    # Lists in a DictConfig are ListConfig (engine.py:20 tests for exactly that);
    # in plain dicts they are Python lists.
    return isinstance(v, list) or type(v).__name__ == "ListConfig"


def _get(d: Any, k: str, default: Any = None) -> Any:
    try:
        return d.get(k, default)
    except AttributeError:
        return getattr(d, k, default)


def initialize_runs(cfg: Any) -> Dict[int, Dict[str, Dict[str, Any]]]:
    """Expand list-valued fields into one run config per sweep point.

    Same contract as src/class/engine.py:13-38: every list in the
    ``exp_type_fp`` and ``physics_fp`` groups is repeated cyclically up to the
    longest list length; a length that does not divide it raises ``ValueError``
    with the reference's message; scalars are shared by all runs.
    """
    groups = (("exp_type_fp", cfg["exp_type_fp"]), ("physics_fp", cfg["physics_fp"]))
    # the swept (list-valued) fields of each group, as plain lists
    sweeps = {name: {k: list(v) for k, v in sub.items() if _is_list(v)} for name, sub in groups}
    n_runs = max((len(v) for sw in sweeps.values() for v in sw.values()), default=1)
    if n_runs == 0:
        return {}
    # every sweep must tile the longest one; the first that does not (in the
    # groups' field order) is reported
    for name, sw in sweeps.items():
        for k, v in sw.items():
            if n_runs % len(v) != 0:
                raise ValueError(f"max_length {n_runs} is not divisible by len({name}.{k})={len(v)}")
    return {i: {name: {k: (sweeps[name][k][i % len(sweeps[name][k])] if k in sweeps[name] else v)
                       for k, v in sub.items()}
                for name, sub in groups}
            for i in range(n_runs)}


def default_config() -> Dict[str, Any]:
    """The reference's default composition of conf/config_fp.yaml: experiment
    group TL12 (conf/exp_type_fp/TL12.yaml) and physics group basicTL12
    (conf/physics_fp/basicTL12.yaml), as plain dicts."""
    return {
        "exp_type_fp": {"name": "TL", "exp_type": "TL", "T_start": [0], "T_end": [1000],
                        "T_rate": [0.1, 1, 5, 20], "duration": [8000, 800, 160, 40], "max_dt": 1,
                        "sims": 2, "holes": 2000, "electrons": 1000, "N_e": 2000, "e_ratio_start": 1,
                        "rho_prime": 3e-4, "boundary_factor": [1.2], "steps": 20000,
                        "distance_plot": False, "x_lim": 800, "bin_size": 1},
        "physics_fp": {"name": "basic", "alpha": 1.6e9, "b": 1e12, "k_b": 8.617343e-5,
                       "E_loc_1": 1.2, "E_loc_2": 1.2, "E_cb": 1000, "D0": 400.35, "D": 0,
                       "Retrap": 0.5, "s": 1e12},
    }
