"""Registry of the compiled device models bundled with the library.

Each model is a MIR + DAE fixture (``<key>.json``) produced by the project's
Verilog-A front end from the reference's bundled ``.va`` sources.  The CUDA
build emits one kernel per fixture; the model id of a key is its index in
sorted key order, which is the order of the library's model table.
"""

from __future__ import annotations

import functools
import json
from dataclasses import dataclass
from pathlib import Path
from typing import Dict, List, Tuple

_DIR = Path(__file__).resolve().parent


@functools.lru_cache(maxsize=None)
def model_keys() -> Tuple[str, ...]:
    return tuple(sorted(p.stem for p in _DIR.glob("*.json")))


@functools.lru_cache(maxsize=None)
def load_model(key: str) -> dict:
    path = _DIR / f"{key}.json"
    if not path.exists():
        raise KeyError(f"unknown device model {key!r}; available: {model_keys()}")
    return json.loads(path.read_text())


@dataclass(frozen=True)
class ModelInfo:
    key: str
    model_id: int
    nodes: Tuple[str, ...]
    terminals: Tuple[str, ...]
    internal: Tuple[str, ...]
    user_params: Tuple[str, ...]
    defaults: Dict[str, float]
    jac: Tuple[Tuple[int, int], ...]
    has_temperature: bool

    def param_index(self, name: str) -> int:
        try:
            return self.user_params.index(name)
        except ValueError:
            low = name.lower()
            for i, p in enumerate(self.user_params):
                if p.lower() == low:
                    return i
            raise KeyError(f"model {self.key}: unknown parameter {name!r}")


@functools.lru_cache(maxsize=None)
def model_info(key: str) -> ModelInfo:
    m = load_model(key)
    nodes = tuple(n["name"] for n in m["dae"]["nodes"])
    user = tuple(n for n, k in zip(m["param_names"], m["param_kinds"]) if k == "param")
    jac = tuple((nodes.index(j["row_node_name"]), nodes.index(j["col_node_name"])) for j in m["dae"]["jacobian"])
    return ModelInfo(
        key=key,
        model_id=model_keys().index(key),
        nodes=nodes,
        terminals=tuple(m["dae"]["terminals"]),
        internal=tuple(m["dae"]["internal_nodes"]),
        user_params=user,
        defaults=dict(m["param_defaults"]),
        jac=jac,
        has_temperature="temperature" in m["param_kinds"],
    )
