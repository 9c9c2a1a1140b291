def record(rec):
    """No-op provenance recorder."""
    return rec
