"""Host-side mirror of GridapMHD's ``main(params)`` / ``hunt(...)`` for the GB300 hot path."""
