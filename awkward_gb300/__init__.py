"""GB300-native kernels for awkward's jagged hot path (placeholder; filled in below)."""
