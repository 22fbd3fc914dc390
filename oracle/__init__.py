"""Parity oracle for the voxplat geometry pipeline (TEST INFRASTRUCTURE ONLY)."""
