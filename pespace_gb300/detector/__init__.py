"""Detector models: orbits, PSDs, TDI data/combination, FD response."""
