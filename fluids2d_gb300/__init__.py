"""fluids2d_gb300: GB300-native time-stepping hot path of Fluids2d."""
