"""Generate the Blosc / zstd / lz4 test fixtures (tests/golden/codecs.npz).

Needs pyarrow (its zstd and raw-LZ4 codecs compress the streams; the tests
only read the .npz). Blosc chunks are assembled here around those streams in
the published Blosc version-1 container layout, in the two forms c-blosc
writes: blocks split into one stream per byte of the type (c-blosc's default
split mode for types of up to 16 bytes) and unsplit blocks; with and without
byte shuffle; several blocks with a partial last block. A small vis.zarr
store written by dio.write_vis is re-encoded with Blosc zstd chunks, the
reference writer's codec (cngi/dio/write_vis.py:62), and stored as
{relative path: file bytes}.

    python tests/golden/make_codec_fixtures.py
"""
import json
import os
import struct
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.abspath(os.path.join(HERE, '..', '..')))

CODE = {'lz4': 1, 'zlib': 3, 'zstd': 4}


def _shuffle(block, typesize):
    n = len(block) // typesize
    head = np.frombuffer(block, dtype=np.uint8, count=n * typesize).reshape(n, typesize).T.reshape(-1)
    return head.tobytes() + block[n * typesize:]


def blosc_chunk(data, typesize, blocksize, compress, codec, shuffle, split):
    """A Blosc version-1 container around streams made by compress(bytes)."""
    nbytes = len(data)
    nblocks = -(-nbytes // blocksize)
    flags = (CODE[codec] << 5) | (0 if split else 0x10) | (0x01 if shuffle else 0)
    base = 16 + 4 * nblocks
    body = bytearray()
    starts = []
    for j in range(nblocks):
        blk = data[j * blocksize:(j + 1) * blocksize]
        last_partial = (nbytes % blocksize) and j == nblocks - 1
        if shuffle and typesize > 1:
            blk = _shuffle(blk, typesize)
        nsplit = typesize if (split and typesize <= 16 and len(blk) // typesize >= 128 and not last_partial) else 1
        ne = len(blk) // nsplit
        starts.append(base + len(body))
        for s in range(nsplit):
            part = blk[s * ne:(s + 1) * ne]
            comp = compress(part)
            if len(comp) >= len(part):
                comp = part                       # stored raw: size == uncompressed size
            body += struct.pack('<i', len(comp)) + comp
    head = struct.pack('<BBBBIII', 2, 1, flags, typesize, nbytes, blocksize, base + len(body))
    return head + struct.pack(f'<{nblocks}i', *starts) + bytes(body)


def main():
    import pyarrow as pa
    from cngi_prototype_gb300 import dio, xds
    rng = np.random.default_rng(5)
    out = {}
    data = {
        'vis': (rng.standard_normal(1500) * 0.3 + 1j * rng.standard_normal(1500) * 0.3).astype(np.complex64),
        'uvw': np.cumsum(rng.standard_normal(1000)).astype(np.float64),
        'flag': (rng.random(6000) < 0.05),
        'text': np.frombuffer(b'the quick brown fox jumps over the lazy dog ' * 150, dtype=np.uint8),
        'zeros': np.zeros(2000, dtype=np.float32),
        'weight': np.where(rng.random(3000) < 0.05, np.nan, 1.0).astype(np.float32),
    }
    for name, arr in data.items():
        raw = arr.tobytes()
        out[f'raw_{name}'] = np.frombuffer(raw, dtype=np.uint8)
        for level in (1, 3, 19):
            c = pa.Codec('zstd', compression_level=level)
            out[f'zstd_{name}_{level}'] = np.frombuffer(c.compress(raw, asbytes=True), dtype=np.uint8)
        out[f'lz4_{name}'] = np.frombuffer(pa.Codec('lz4_raw').compress(raw, asbytes=True), dtype=np.uint8)
    # Blosc chunks
    zc = pa.Codec('zstd', compression_level=2)
    lz = pa.Codec('lz4_raw')
    import zlib
    comps = {'zstd': lambda b: zc.compress(b, asbytes=True), 'lz4': lambda b: lz.compress(b, asbytes=True),
             'zlib': lambda b: zlib.compress(b, 5)}
    for name, ts in (('vis', 8), ('weight', 4), ('text', 1)):
        raw = data[name].tobytes()
        for codec, variants in (('zstd', ((False, False), (False, True), (True, False), (True, True))),
                                ('lz4', ((False, True), (True, False))), ('zlib', ((True, True),))):
            for shuffle, split in variants:
                for bs in (2048, len(raw)):
                    out[f'blosc_{name}_{codec}_{int(shuffle)}{int(split)}_{bs}'] = np.frombuffer(
                        blosc_chunk(raw, ts, bs, comps[codec], codec, shuffle, split), dtype=np.uint8)
    # a vis.zarr store with Blosc(zstd, clevel 2, no shuffle) chunks
    T, B, C, P = 6, 10, 4, 2
    uvw = rng.standard_normal((T, B, 3)) * 300
    vis = (rng.standard_normal((T, B, C, P)) + 1j * rng.standard_normal((T, B, C, P))).astype(np.complex64)
    w = rng.uniform(0.5, 2, (T, B, C, P)).astype(np.float32)
    fl = rng.random((T, B, C, P)) < 0.1
    vds = xds.vis_dataset(uvw, vis, w, 1e9 + 1e6 * np.arange(C), flag=fl)
    mx = xds.mxds({'xds0': vds})
    with tempfile.TemporaryDirectory() as tmp:
        store = os.path.join(tmp, 's.vis.zarr')
        dio.write_vis(mx, store, chunks_on_disk={'time': 4, 'chan': 3})
        for root, _, files in os.walk(store):
            for f in files:
                p = os.path.join(root, f)
                rel = os.path.relpath(p, store)
                b = open(p, 'rb').read()
                if f == '.zarray':
                    meta = json.loads(b)
                    meta['compressor'] = {'id': 'blosc', 'cname': 'zstd', 'clevel': 2, 'shuffle': 0,
                                          'blocksize': 0}
                    b = json.dumps(meta).encode()
                elif f == '.zmetadata':
                    md = json.loads(b)
                    for key, v in md['metadata'].items():
                        if key.endswith('/.zarray'):
                            v['compressor'] = {'id': 'blosc', 'cname': 'zstd', 'clevel': 2, 'shuffle': 0,
                                               'blocksize': 0}
                    b = json.dumps(md).encode()
                elif not f.startswith('.'):
                    meta = json.load(open(os.path.join(root, '.zarray')))
                    ts = np.dtype(meta['dtype']).itemsize
                    b = blosc_chunk(b, ts, max(len(b), 1), comps['zstd'], 'zstd', False, True)
                out['store/' + rel] = np.frombuffer(b, dtype=np.uint8)
    out['store_vis'] = vis
    out['store_uvw'] = uvw
    out['store_weight'] = w
    out['store_flag'] = fl
    np.savez_compressed(os.path.join(HERE, 'codecs.npz'), **out)
    print(len(out), 'entries', os.path.getsize(os.path.join(HERE, 'codecs.npz')), 'bytes')


if __name__ == '__main__':
    main()
