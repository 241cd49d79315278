"""Blosc, zstd (RFC 8878) and LZ4 decoding for vis.zarr stores written with
the reference's codec (Blosc zstd, cngi/dio/write_vis.py:62), against streams
made by an independent compressor (tests/golden/make_codec_fixtures.py) and
hand-assembled frames."""
import os
import struct

import numpy as np
import pytest

from conftest import load_golden
from cngi_prototype_gb300 import _blosc, _zstd, dio


@pytest.fixture(scope='module')
def fx():
    return load_golden('codecs')


def test_xxh64_published_vectors():
    assert _zstd.xxh64(b'') == 0xEF46DB3751D8E999
    assert _zstd.xxh64(b'a') == 0xD24EC4F1A98C6E5B
    assert _zstd.xxh64(b'abc') == 0x44BC2CF5AD770999
    assert _zstd.xxh64(b'Nobody inspects the spammish repetition') == 0xFBCEA83C8A378BF1


def test_zstd_frames_decode(fx):
    keys = [k for k in fx if k.startswith('zstd_')]
    assert len(keys) == 18
    for k in keys:
        name = k.split('_')[1]
        assert _zstd.decompress(fx[k].tobytes()) == fx['raw_' + name].tobytes(), k


def test_zstd_hand_assembled_frames():
    """Raw and RLE blocks, a single-segment header, a checksum, a skippable
    frame and two concatenated frames."""
    payload = b'radio interferometry'
    ck = (_zstd.xxh64(payload) & 0xFFFFFFFF).to_bytes(4, 'little')
    raw_block = (1 | (0 << 1) | (len(payload) << 3)).to_bytes(3, 'little') + payload
    # single segment (bit 5), content size in 1 byte, checksum (bit 2)
    f1 = struct.pack('<I', 0xFD2FB528) + bytes([0x24, len(payload)]) + raw_block + ck
    assert _zstd.decompress(f1) == payload
    rle = (1 | (1 << 1) | (1000 << 3)).to_bytes(3, 'little') + b'\x07'
    f2 = struct.pack('<I', 0xFD2FB528) + bytes([0x00, 0x40]) + rle     # window descriptor, no content size
    skip = struct.pack('<II', 0x184D2A53, 3) + b'xyz'
    assert _zstd.decompress(f1 + skip + f2) == payload + b'\x07' * 1000
    bad = f1[:-1] + bytes([f1[-1] ^ 1])
    with pytest.raises(_zstd.ZstdError, match='checksum'):
        _zstd.decompress(bad)
    with pytest.raises(_zstd.ZstdError):
        _zstd.decompress(b'\x00\x01\x02\x03\x04')


def test_lz4_blocks_decode(fx):
    for k in [k for k in fx if k.startswith('lz4_')]:
        raw = fx['raw_' + k.split('_')[1]].tobytes()
        assert _blosc._lz4_block(fx[k].tobytes(), len(raw)) == raw, k


def test_blosc_chunks_decode(fx):
    keys = [k for k in fx if k.startswith('blosc_')]
    assert len(keys) == 42
    for k in keys:
        name = k.split('_')[1]
        assert _blosc.decompress(fx[k].tobytes()) == fx['raw_' + name].tobytes(), k


def test_blosc_stored_and_refused_forms():
    data = bytes(range(200)) * 3
    memcpyed = struct.pack('<BBBBIII', 2, 1, 0x02 | (4 << 5), 1, len(data), len(data), 16 + len(data)) + data
    assert _blosc.decompress(memcpyed) == data
    # one block whose stream is stored raw (size == uncompressed size)
    one = struct.pack('<BBBBIII', 2, 1, 0x10 | (4 << 5), 1, len(data), len(data), 24 + len(data))
    one += struct.pack('<i', 20) + struct.pack('<i', len(data)) + data
    assert _blosc.decompress(one) == data
    bitshuffle = struct.pack('<BBBBIII', 2, 1, 0x04 | (4 << 5), 4, 8, 8, 24) + bytes(8)
    with pytest.raises(NotImplementedError, match='bit shuffle'):
        _blosc.decompress(bitshuffle)
    snappy = struct.pack('<BBBBIII', 2, 1, 0x10 | (2 << 5), 1, 8, 8, 28) + struct.pack('<ii', 20, 4) + b'abcd'
    with pytest.raises(NotImplementedError, match='snappy'):
        _blosc.decompress(snappy)


def test_read_vis_of_a_blosc_zstd_store(fx, tmp_path):
    """A store whose every array is Blosc(cname='zstd', clevel=2, shuffle=0)
    compressed, the reference writer's codec, reads back exactly."""
    store = tmp_path / 's.vis.zarr'
    for k in fx:
        if not k.startswith('store/'):
            continue
        p = store / k[len('store/'):]
        os.makedirs(p.parent, exist_ok=True)
        p.write_bytes(fx[k].tobytes())
    mx = dio.read_vis(str(store))
    v = mx.attrs['xds0']
    assert np.array_equal(v['DATA'].values, fx['store_vis'])
    assert np.array_equal(v['UVW'].values, fx['store_uvw'])
    assert np.array_equal(v['DATA_WEIGHT'].values, fx['store_weight'])
    assert np.array_equal(v['FLAG'].values, fx['store_flag'])
