"""Blosc (version 1 format) chunk decompression, pure Python.

The reference writes every vis.zarr array with numcodecs'
Blosc(cname='zstd', clevel=2, shuffle=0) (cngi/dio/write_vis.py:62,
cngi/dio/append_xds.py:69); numcodecs is not available here, so the
container is decoded from the published Blosc format:

* a 16-byte header: format version, codec format version, flags (bit 0
  byte shuffle, bit 1 stored uncompressed, bit 2 bit shuffle, bit 4 blocks
  not split into per-byte streams, bits 5-7 the codec: 0 blosclz, 1 lz4,
  2 snappy, 3 zlib, 4 zstd), type size, then uncompressed size, block size
  and compressed size as little-endian uint32;
* unless stored uncompressed, one int32 start offset per block, and at each
  block its streams (one, or one per byte of the type when the block is
  split), each an int32 compressed size followed by its bytes (stored raw
  when that size equals the stream's uncompressed size);
* byte shuffle undone per block (the bytes of equal significance of the
  block's items are stored together).

Codecs decoded: zstd (this package's RFC 8878 decoder), zlib and lz4;
blosclz, snappy and bit shuffle raise NotImplementedError.
"""
import struct
import zlib

import numpy as np

from . import _zstd

_CODECS = {0: 'blosclz', 1: 'lz4', 2: 'snappy', 3: 'zlib', 4: 'zstd'}
MAX_SPLITS = 16          # blocks of types up to 16 bytes may be split per byte
MIN_BUFFERSIZE = 128     # ... when each split stream holds at least this many bytes


class BloscError(ValueError):
    """Malformed Blosc data."""


def _lz4_block(src, n_out):
    """LZ4 block format: tokens of literal and match lengths, 16-bit offsets."""
    out = bytearray()
    p = 0
    end = len(src)
    while p < end:
        tok = src[p]
        p += 1
        ll = tok >> 4
        if ll == 15:
            while True:
                b = src[p]
                p += 1
                ll += b
                if b != 255:
                    break
        out += src[p:p + ll]
        p += ll
        if p >= end:
            break
        off = src[p] | (src[p + 1] << 8)
        p += 2
        ml = tok & 15
        if ml == 15:
            while True:
                b = src[p]
                p += 1
                ml += b
                if b != 255:
                    break
        ml += 4
        if off == 0 or off > len(out):
            raise BloscError('lz4 match offset outside the block')
        start = len(out) - off
        if off >= ml:
            out += out[start:start + ml]
        else:
            chunk = bytes(out[start:])
            reps, r = divmod(ml, off)
            out += chunk * reps + chunk[:r]
    if len(out) != n_out:
        raise BloscError(f'lz4 block gave {len(out)} bytes, expected {n_out}')
    return bytes(out)


def _decode_stream(codec, data, n_out):
    if codec == 'zstd':
        out = _zstd.decompress(data)
    elif codec == 'zlib':
        out = zlib.decompress(data)
    elif codec == 'lz4':
        out = _lz4_block(data, n_out)
    else:
        raise NotImplementedError(f'Blosc codec {codec!r} is not supported (zstd, zlib and lz4 are)')
    if len(out) != n_out:
        raise BloscError(f'{codec} stream gave {len(out)} bytes, expected {n_out}')
    return out


def _unshuffle(block, typesize):
    n = len(block) // typesize
    head = np.frombuffer(block, dtype=np.uint8, count=n * typesize).reshape(typesize, n).T.reshape(-1)
    return head.tobytes() + block[n * typesize:]


def header(buf):
    """(version, codec version, flags, typesize, nbytes, blocksize, cbytes)."""
    if len(buf) < 16:
        raise BloscError('Blosc buffer shorter than its header')
    return struct.unpack_from('<BBBBIII', buf, 0)


def decompress(buf):
    """Decompress one Blosc chunk (bytes in, bytes out)."""
    buf = bytes(buf)
    version, _, flags, typesize, nbytes, blocksize, cbytes = header(buf)
    if version not in (1, 2):
        raise NotImplementedError(f'Blosc format version {version} (only the version-1/2 container is supported)')
    if cbytes > len(buf):
        raise BloscError(f'Blosc chunk truncated: {len(buf)} of {cbytes} bytes')
    if flags & 0x02:
        return buf[16:16 + nbytes]
    if flags & 0x04:
        raise NotImplementedError('Blosc bit shuffle is not supported')
    if nbytes == 0:
        return b''
    if blocksize == 0 or typesize == 0:
        raise BloscError('Blosc header with a zero block or type size')
    codec = _CODECS.get(flags >> 5)
    if codec is None:
        raise BloscError(f'unknown Blosc codec code {flags >> 5}')
    dont_split = bool(flags & 0x10)
    nblocks = -(-nbytes // blocksize)
    leftover = nbytes % blocksize
    starts = struct.unpack_from(f'<{nblocks}i', buf, 16)
    out = bytearray()
    for j, st in enumerate(starts):
        last_partial = leftover and j == nblocks - 1
        bsize = leftover if last_partial else blocksize
        split = (not dont_split and typesize <= MAX_SPLITS and bsize // typesize >= MIN_BUFFERSIZE
                 and not last_partial)
        nsplits = typesize if split else 1
        neblock = bsize // nsplits
        p = st
        block = bytearray()
        for _ in range(nsplits):
            cb = struct.unpack_from('<i', buf, p)[0]
            p += 4
            if cb == neblock:
                block += buf[p:p + cb]
            else:
                block += _decode_stream(codec, buf[p:p + cb], neblock)
            p += cb
        if len(block) != bsize:
            raise BloscError(f'Blosc block {j}: {len(block)} bytes, expected {bsize}')
        if flags & 0x01 and typesize > 1:
            block = _unshuffle(bytes(block), typesize)
        out += block
    return bytes(out)
