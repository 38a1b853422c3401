"""Symbolic parameter paths (tree_utils.py:34-122, 168-180).

``component.params.focal_length`` (or ``ray.params.x``,
``descanner.params.descan_error.pxo_pxi``) is a ``PathBuilder``: a record of
the object it starts from and the attribute / item keys below it.
``run_with_grads`` takes a list of them to choose what to differentiate.
"""
from __future__ import annotations

import dataclasses
from types import SimpleNamespace
from typing import Any


class PathBuilder:
    """A path from a root object through attribute ("attr") or item ("item")
    keys (tree_utils.py:34-122)."""

    def __init__(self, parent: Any, key, getter: str):
        if getter not in ("attr", "item"):
            raise ValueError(f"Unknown get with {getter}")
        object.__setattr__(self, "_parent", parent)
        object.__setattr__(self, "_original_key", key)
        object.__setattr__(self, "_getter", getter)
        true_parent = self._resolve_parent()
        if not (dataclasses.is_dataclass(true_parent) or isinstance(true_parent, (list, tuple, dict))
                or hasattr(true_parent, "_fields")):
            raise NotImplementedError(f"Unknown key type for cls {type(true_parent)}")

    def __getattr__(self, name: str):
        if name.startswith("__"):
            raise AttributeError(name)
        return type(self)(self, name, "attr")

    def __getitem__(self, idx):
        return type(self)(self, idx, "item")

    def __repr__(self):
        keys = self._build()[1:]
        return f"PathBuilder({type(self._resolve_root()).__name__}" + "".join(f".{k}" for k in keys) + ")"

    def _resolve_root(self):
        p = self._parent
        return p._resolve_root() if isinstance(p, PathBuilder) else p

    def _resolve_parent(self):
        p = self._parent
        return p._resolve() if isinstance(p, PathBuilder) else p

    def _resolve(self):
        src = self._resolve_parent()
        if self._getter == "attr":
            return getattr(src, self._original_key)
        return src[self._original_key]

    def _build(self, children: tuple = (), original: bool = True) -> tuple:
        """(root, key, key, ...).  Keys are the attribute names / indices as
        written (the reference's ``original=True`` form; ``original`` is
        accepted for signature compatibility)."""
        this = (self._original_key,) + tuple(children)
        if isinstance(self._parent, PathBuilder):
            return self._parent._build(this, original)
        return (self._parent,) + this


class HasParamsMixin:
    """``obj.params.<field>`` gives a PathBuilder rooted at ``obj``
    (tree_utils.py:168-180)."""

    @property
    def params(self):
        names = [f.name for f in dataclasses.fields(self)]
        return SimpleNamespace(**{n: PathBuilder(self, n, "attr") for n in names})

    def new_with(self, **kwargs):
        return dataclasses.replace(self, **kwargs)


def isnamedtuple(obj) -> bool:
    """tree_utils.py:14-19."""
    return isinstance(obj, tuple) and hasattr(obj, "_asdict") and hasattr(obj, "_fields")
