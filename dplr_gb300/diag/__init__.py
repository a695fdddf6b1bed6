"""Diagnostics: hardware peak probes used as roofline denominators."""
