"""GB300-native phase linking: a drop-in for dolphin's phase-linking hot path."""
