"""sparqc_gb300: GB300-native sparse statevector gate engine."""
