"""xcorr_gb300: Python binding of the GB300 xcorr library (placeholder, filled in below)."""
