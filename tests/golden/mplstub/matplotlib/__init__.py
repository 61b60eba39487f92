"""Minimal stand-in for matplotlib so that the reference package can be imported
without a plotting stack. Only used by the golden-vector generator; nothing here draws."""
