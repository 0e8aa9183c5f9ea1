"""pibiti_gb300: a GB300-native SPH simulation step."""
