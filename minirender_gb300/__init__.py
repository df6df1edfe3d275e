"""GB300 (sm_103a) rasterisation path behind minirender's Renderer API."""
