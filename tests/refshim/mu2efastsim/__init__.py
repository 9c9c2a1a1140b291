"""Test-only stand-in for the reference's core package (only the pieces its CRV response modules import)."""
