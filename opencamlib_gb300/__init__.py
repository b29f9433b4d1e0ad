"""opencamlib_gb300 -- GB300-native drop-cutter / push-cutter (placeholder; binding follows)."""
