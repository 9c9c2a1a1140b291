"""Test-only stand-in for pandas, which is not installed here.

The reference coincidence module imports pandas at module level but only touches it in its optional
"reference" attachment mode; the default NumPy attachment mode never does. Any use raises.
"""


class DataFrame:  # pragma: no cover - never constructed in the modes the golden generator uses
    def __init__(self, *a, **k):
        raise RuntimeError("pandas is not available in this environment")
