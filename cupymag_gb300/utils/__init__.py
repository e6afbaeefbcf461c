"""Subpackage of cupymag_gb300."""
