"""GB300-native Newton step for Rismo2D's depth-averaged shallow-water equations."""
