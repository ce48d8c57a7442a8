"""Result comparison with the reference's tolerances.

Same rule as stencil_benchmarks/tools/validation.py:98-116: ``np.isclose``
with rtol 1e-4 / atol 1e-5 for float32 and numpy's defaults (rtol 1e-5,
atol 1e-8) otherwise; a failure raises ``ValidationError`` listing the first
failing points.  bfloat16 fields (held as uint16 bit patterns) are widened to
float32 and compared with rtol 1e-2 / atol 1e-2 (bfloat16 has 8 significant
bits).
"""

from __future__ import annotations

import numpy as np


class ValidationError(RuntimeError):
    """A field differs from its expected value (the CLI exits with status 2)."""


def bf16_to_f32(bits: np.ndarray) -> np.ndarray:
    """Widen bfloat16 bit patterns (uint16) to float32 exactly."""
    return (np.ascontiguousarray(bits, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32).reshape(
        np.shape(bits))


def tolerances(dtype, storage: str | None = None):
    if storage == "bfloat16":
        return {"rtol": 1e-2, "atol": 1e-2}
    if np.dtype(dtype) == np.float32:
        return {"rtol": 1e-4, "atol": 1e-5}
    return {}


def check_equality(name: str, result: np.ndarray, expected: np.ndarray, storage: str | None = None):
    if storage == "bfloat16":
        result, expected = bf16_to_f32(result), bf16_to_f32(expected)
    if result.dtype != expected.dtype:
        raise ValidationError(f"field {name}: dtype {result.dtype} differs from expected {expected.dtype}")
    failure = ~np.isclose(result, expected, **tolerances(result.dtype, storage))
    if not np.any(failure):
        return
    idx = np.argwhere(failure)
    lines = [f"validation of field {name} failed at {len(idx)} points:"]
    for p in idx[:20]:
        p = tuple(int(x) for x in p)
        lines.append(f"failed at {p}: {result[p]!r} != {expected[p]!r}")
    if len(idx) > 20:
        lines.append(f"omitted further {len(idx) - 20} failures.")
    raise ValidationError("\n".join(lines))
