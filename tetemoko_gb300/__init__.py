"""GB300-native per-level Godunov step of tetemoko (2-D elastic rupture)."""
from . import _capi  # noqa: F401
