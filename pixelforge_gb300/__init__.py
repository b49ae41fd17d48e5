"""pixelforge-gb300: PixelForge's triangle pipeline on a GB300 (sm_103a)."""
