"""Command-line drop-ins for kore's scripts."""
