"""Test-only empty stand-in for ``matplotlib.pyplot``; plotting is never called."""
