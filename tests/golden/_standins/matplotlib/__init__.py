"""Test-only empty stand-in for ``matplotlib`` (absent in this container)."""
