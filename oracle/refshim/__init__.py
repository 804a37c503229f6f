"""Test infrastructure: runs the reference's own UPPE path on host cores to make golden fixtures."""
