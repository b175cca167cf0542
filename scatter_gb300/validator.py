"""Load dictionary validation: drop-in for scatter/validator.py (same checks and defaults)."""
from typing import Dict

LOAD_TYPES = ("pulse", "heaviside", "moving", "moving_at_plane", "rose")


class ValidateLoad:
    @staticmethod
    def validate(loading: Dict):
        """Asserts ``type`` and sets ``ini_steps`` to 5 when absent (validator.py:34-57)."""
        assert "type" in loading
        if loading["type"] not in LOAD_TYPES:
            raise Exception(f'Error: Load type {loading["type"]} not supported')
        loading.setdefault("ini_steps", 5)
