"""Benchmark / Parameter API, the same contract as the reference's.

Mirrors stencil_benchmarks/benchmark.py:33-220 so that backends written
against the reference's interface work here unchanged:

* ``Parameter(description, default=None, dtype=None, nargs=None, choices=None)``
  declares a typed knob; a missing default makes it required.
* Subclasses of ``Benchmark`` collect the Parameters of their bases and their
  own class body into ``cls.parameters``; every class that is not abstract is
  added to ``REGISTRY``.
* ``Benchmark(**kwargs)`` validates every argument (``ParameterError`` on a bad
  one, ``ValueError`` on an unknown name) and calls ``setup()``; assigning a
  parameter later re-validates it; ``run()`` / ``__call__`` return a dict or a
  list of dicts with at least a ``time`` key.
"""

from __future__ import annotations

import abc
import inspect
from typing import Any, Dict, Iterable, List, Optional, Type, Union

REGISTRY = set()


class ParameterError(ValueError):
    """An argument failed validation (the CLI skips such configurations with -s)."""


class ExecutionError(RuntimeError):
    """A benchmark failed while running (the CLI skips it with -q)."""


class Parameter:
    def __init__(
        self,
        description: str,
        default: Any = None,
        dtype: Optional[Type] = None,
        nargs: Optional[int] = None,
        choices: Optional[Iterable] = None,
    ):
        if default is None:
            if dtype is None or nargs is None:
                raise ValueError("a parameter without default needs dtype and nargs")
        else:
            if isinstance(default, (tuple, list)):
                if not default:
                    raise ValueError("an empty tuple can not be a default")
                types = {type(d) for d in default}
                if len(types) > 1:
                    raise ValueError("mixed types in a default tuple")
                implied_dtype, implied_nargs = types.pop(), len(default)
            else:
                implied_dtype, implied_nargs = type(default), 1
            if dtype is None:
                dtype = implied_dtype
            elif dtype is not implied_dtype:
                raise ValueError("default does not match dtype")
            if nargs is None:
                nargs = implied_nargs
            elif nargs != implied_nargs:
                raise ValueError("default does not match nargs")
        self.description = description
        self.default = default
        self.dtype = dtype
        self.nargs = nargs
        self.choices = tuple(choices) if choices is not None else None

    def validate(self, value):
        if value is None:
            if self.default is None:
                raise ParameterError("value is required")
            value = self.default
        if self.nargs == 1:
            if not isinstance(value, self.dtype):
                raise ParameterError(
                    f'wrong type of argument "{value}", expected one of type "{self.dtype.__name__}"'
                )
        else:
            if not isinstance(value, (tuple, list)):
                raise ParameterError(
                    f'{self.nargs} arguments of type "{self.dtype.__name__}" required, found "{value}"'
                )
            if len(value) != self.nargs:
                raise ParameterError(f'wrong number of arguments in argument "{value}"')
            if not all(isinstance(v, self.dtype) for v in value):
                raise ParameterError(f'wrong type in argument "{value}"')
        if self.choices is not None and value not in self.choices:
            options = ", ".join(f'"{c}"' for c in self.choices)
            raise ParameterError(f'unsupported argument value "{value}", choices are {options}')
        return value

    def __repr__(self):
        return (
            f"{type(self).__name__}(description={self.description!r}, dtype={self.dtype!r}, "
            f"nargs={self.nargs!r}, default={self.default!r})"
        )

    def __eq__(self, other):
        return (
            self.description == other.description
            and self.dtype is other.dtype
            and self.nargs == other.nargs
            and self.default == other.default
        )

    __hash__ = None


class BenchmarkMeta(abc.ABCMeta):
    def __new__(mcs, name, bases, namespace):
        if "parameters" in namespace:
            raise AttributeError("Benchmark classes must not define an attribute `parameters`")
        parameters = {}
        for base in bases:
            parameters.update(getattr(base, "parameters", {}))
        body = {}
        for key, value in namespace.items():
            if isinstance(value, Parameter):
                parameters[key] = value
            else:
                body[key] = value
        body["parameters"] = parameters
        cls = super().__new__(mcs, name, bases, body)
        if not inspect.isabstract(cls):
            REGISTRY.add(cls)
        return cls


class Benchmark(metaclass=BenchmarkMeta):
    def __init__(self, **kwargs):
        unknown = set(kwargs) - set(self.parameters)
        if unknown:
            raise ValueError("unsupported arguments " + ", ".join(f'"{a}"' for a in sorted(unknown)))
        values = {}
        for name, param in self.parameters.items():
            try:
                values[name] = param.validate(kwargs.get(name))
            except ParameterError as err:
                raise ParameterError(f'invalid value for argument "{name}": ' + err.args[0]) from None
        self.parameters = values
        self.setup()

    def __setattr__(self, name: str, value):
        if name in self.parameters:
            self.parameters[name] = type(self).parameters[name].validate(value)
        else:
            super().__setattr__(name, value)

    def __getattr__(self, name: str):
        params = self.__dict__.get("parameters")
        if params is not None and name in params:
            return params[name]
        raise AttributeError(f"{type(self).__name__!r} object has no attribute {name!r}")

    def setup(self) -> None:
        """Prepare the benchmark (called once by the constructor)."""

    @abc.abstractmethod
    def run(self) -> Union[Dict[str, Any], List[Dict[str, Any]]]:
        """Run once and return the timing result(s)."""

    def __call__(self):
        return self.run()

    def __repr__(self) -> str:
        args = ", ".join(f"{k}={v!r}" for k, v in self.parameters.items())
        return f"{type(self).__name__}({args})"
