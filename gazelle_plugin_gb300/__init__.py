"""GB300-native columnar shuffle hash split (drop-in for Gazelle's native HashSplitter)."""
