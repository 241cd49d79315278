"""Helpers behind the ngcasa.imaging-compatible API (kernel tables, parameter
checks, and the per-chunk gridding functions the reference's graph builders
call, here backed by libngg)."""
