"""Builds and launchers of the reference's own code (test infrastructure)."""
