from . import gb300

__all__ = ["gb300"]
