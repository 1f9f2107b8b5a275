"""Loader for the golden fixtures written by ``make_golden.py``."""

from __future__ import annotations

import functools
import json
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class Case:
    def __init__(self, store: "Store", name: str):
        self._s = store
        self.name = name
        self.meta = store.meta.get(name, {})

    def __getitem__(self, key: str) -> np.ndarray:
        return self._s.data[f"{self.name}/{key}"]

    def has(self, key: str) -> bool:
        return f"{self.name}/{key}" in self._s.data.files

    def tuple(self, key: str) -> tuple[np.ndarray, ...]:
        n = self.meta[f"{key}_len"]
        return tuple(self[f"{key}_{k}"] for k in range(n))

    def weights(self, key: str = "weights"):
        """The saved-layout triple ``(object array, shape_input, shape_output)``."""
        m = self.meta[key]
        shape = tuple(m["shape"])
        n = int(np.prod(shape)) if shape else 1
        flat = np.empty(n, dtype=object)
        for k in range(n):
            flat[k] = (self[f"{key}_{k}_in"], self[f"{key}_{k}_out"], self[f"{key}_{k}_val"])
        return flat.reshape(shape), tuple(m["shape_input"]), tuple(m["shape_output"])


class Store:
    def __init__(self, path: str):
        self.data = np.load(path, allow_pickle=False)
        self.meta = json.loads(str(self.data["__meta__"]))

    def case(self, name: str) -> Case:
        return Case(self, name)

    def names(self, prefix: str = "") -> list[str]:
        return sorted(k for k in self.meta if k.startswith(prefix))


@functools.lru_cache(maxsize=None)
def load(name: str) -> Store:
    return Store(os.path.join(HERE, name))
