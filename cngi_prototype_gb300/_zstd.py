"""Zstandard decompression (RFC 8878), pure Python.

The chunk codec of the reference's vis.zarr stores is Blosc with the zstd
compressor (cngi/dio/write_vis.py:62, Blosc(cname='zstd', clevel=2,
shuffle=0)); numcodecs is not available on these machines, so the format is
decoded here from its specification: frames (and skippable frames), raw,
RLE and compressed blocks; literals sections (raw, RLE, Huffman-coded with
one or four streams, with a new or the previous Huffman table); sequences
sections with predefined, RLE, FSE-coded and repeated tables; the repeat
offsets; the frame content size and the XXH64 content checksum. Dictionaries
are not supported (the reference's writers use none).

Decoding is sequential bit-level work, so this runs at a few MB/s: enough
to read stores in tests and small observations; large stores are read
chunk by chunk.
"""


class ZstdError(ValueError):
    """Malformed or unsupported zstd data."""


_MAGIC = 0xFD2FB528

# ---- RFC 8878 3.1.1.3.2.1: codes, baselines and extra bits -----------------
_LL_BASE = list(range(16)) + [16, 18, 20, 22, 24, 28, 32, 40, 48, 64, 128, 256, 512, 1024, 2048, 4096, 8192,
                              16384, 32768, 65536]
_LL_BITS = [0] * 16 + [1, 1, 1, 1, 2, 2, 3, 3, 4, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16]
_ML_BASE = [c + 3 for c in range(32)] + [35, 37, 39, 41, 43, 47, 51, 59, 67, 83, 99, 131, 259, 515, 1027, 2051,
                                         4099, 8195, 16387, 32771, 65539]
_ML_BITS = [0] * 32 + [1, 1, 1, 1, 2, 2, 3, 3, 4, 4, 5, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16]

# ---- RFC 8878 3.1.1.3.2.2: predefined distributions ------------------------
_LL_DEFAULT = ([4, 3, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 2, 1, 1, 1, 2, 2, 2, 2, 2, 2, 2, 2, 2, 3, 2, 1, 1, 1, 1, 1,
                -1, -1, -1, -1], 6)
_ML_DEFAULT = ([1, 4, 3, 2, 2, 2, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1,
                1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1, -1, -1], 6)
_OF_DEFAULT = ([1, 1, 1, 1, 1, 1, 2, 2, 2, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, 1, -1, -1, -1, -1, -1], 5)


class _BackBits:
    """Backward bit stream: the bytes form one little-endian integer whose
    highest set bit is a start marker; bits are consumed from just below the
    marker towards bit 0. Bits below 0 read as zeros (and mark an overflow)."""
    __slots__ = ('d', 'pos')

    def __init__(self, data):
        if not data or data[-1] == 0:
            raise ZstdError('backward bit stream without its end marker')
        self.d = data
        self.pos = (len(data) - 1) * 8 + data[-1].bit_length() - 1

    def peek(self, n):
        if n == 0:
            return 0
        p = self.pos - n
        if p >= 0:
            b0 = p >> 3
            x = int.from_bytes(self.d[b0:(self.pos + 7) >> 3], 'little') >> (p & 7)
            return x & ((1 << n) - 1)
        if self.pos <= 0:
            return 0
        x = int.from_bytes(self.d[0:(self.pos + 7) >> 3], 'little') & ((1 << self.pos) - 1)
        return x << (-p)

    def read(self, n):
        v = self.peek(n)
        self.pos -= n
        return v


class _FwdBits:
    """Forward little-endian bit reader (FSE table descriptions)."""
    __slots__ = ('d', 'start', 'bit')

    def __init__(self, data, start):
        self.d = data
        self.start = start
        self.bit = 0

    def peek(self, n):
        b = self.start * 8 + self.bit
        b0 = b >> 3
        x = int.from_bytes(self.d[b0:b0 + ((b & 7) + n + 7) // 8], 'little') >> (b & 7)
        return x & ((1 << n) - 1)

    def read(self, n):
        v = self.peek(n)
        self.bit += n
        return v

    def nbytes(self):
        return (self.bit + 7) >> 3


# ---- FSE (RFC 8878 4.1) -------------------------------------------------------
def _read_distribution(data, pos, max_symbols, max_log):
    """An FSE table description: (normalized counts, accuracy log, bytes used)."""
    br = _FwdBits(data, pos)
    acc = br.read(4) + 5
    if acc > max_log:
        raise ZstdError(f'FSE accuracy log {acc} above {max_log}')
    size = 1 << acc
    remaining = size + 1
    threshold = size
    nbits = acc + 1
    counts = []
    while remaining > 1 and len(counts) < max_symbols:
        mx = 2 * threshold - 1 - remaining
        low = br.peek(nbits - 1)
        if low < mx:
            value = low
            br.bit += nbits - 1
        else:
            value = br.peek(nbits)
            if value >= threshold:
                value -= mx
            br.bit += nbits
        c = value - 1
        counts.append(c)
        remaining -= -c if c < 0 else c
        if c == 0:
            while True:
                rep = br.read(2)
                counts.extend([0] * rep)
                if rep != 3:
                    break
        while remaining < threshold:
            nbits -= 1
            threshold >>= 1
    if remaining != 1 or len(counts) > max_symbols:
        raise ZstdError('corrupt FSE table description')
    return counts, acc, br.nbytes()


def _fse_table(counts, acc):
    """Decoding table (symbol, bits, baseline per state) of a distribution."""
    size = 1 << acc
    sym = [0] * size
    high = size - 1
    nxt = [0] * len(counts)
    for s, c in enumerate(counts):
        if c == -1:
            sym[high] = s
            high -= 1
            nxt[s] = 1
        else:
            nxt[s] = c
    step = (size >> 1) + (size >> 3) + 3
    mask = size - 1
    p = 0
    for s, c in enumerate(counts):
        for _ in range(c if c > 0 else 0):
            sym[p] = s
            p = (p + step) & mask
            while p > high:
                p = (p + step) & mask
    if p != 0:
        raise ZstdError('FSE distribution does not fill its table')
    nb = [0] * size
    base = [0] * size
    for u in range(size):
        s = sym[u]
        ns = nxt[s]
        nxt[s] += 1
        k = acc - (ns.bit_length() - 1)
        nb[u] = k
        base[u] = (ns << k) - size
    return sym, nb, base, acc


_TABLES = {}


def _default_table(which):
    if which not in _TABLES:
        counts, acc = {'ll': _LL_DEFAULT, 'ml': _ML_DEFAULT, 'of': _OF_DEFAULT}[which]
        _TABLES[which] = _fse_table(counts, acc)
    return _TABLES[which]


# ---- Huffman literals (RFC 8878 4.2) -------------------------------------------
def _huffman_table(data, pos):
    """Huffman tree description at pos: (decoding table, max bits, bytes used)."""
    hb = data[pos]
    if hb < 128:
        src = data[pos + 1:pos + 1 + hb]
        counts, acc, used = _read_distribution(src, 0, 256, 6)
        sym, nb, base, acc = _fse_table(counts, acc)
        br = _BackBits(src[used:])
        s1 = br.read(acc)
        s2 = br.read(acc)
        weights = []
        while len(weights) < 255:
            weights.append(sym[s1])
            s1 = base[s1] + br.read(nb[s1])
            if br.pos < 0:
                weights.append(sym[s2])
                break
            weights.append(sym[s2])
            s2 = base[s2] + br.read(nb[s2])
            if br.pos < 0:
                weights.append(sym[s1])
                break
        used_total = 1 + hb
    else:
        n = hb - 127
        nbytes = (n + 1) // 2
        weights = [(data[pos + 1 + i // 2] >> 4) if i % 2 == 0 else (data[pos + 1 + i // 2] & 15) for i in range(n)]
        used_total = 1 + nbytes
    total = sum(1 << (w - 1) for w in weights if w > 0)
    if total == 0:
        raise ZstdError('empty Huffman weights')
    maxbits = total.bit_length()
    rest = (1 << maxbits) - total
    if rest & (rest - 1):
        raise ZstdError('Huffman weights do not complete a power of two')
    weights.append(rest.bit_length())
    if maxbits > 11:
        raise ZstdError('Huffman code longer than 11 bits')
    # canonical table: weight-1 symbols first (one cell each), then weight 2, ...
    rank = [0] * (maxbits + 2)
    for w in weights:
        if w:
            rank[w] += 1
    start = [0] * (maxbits + 2)
    acc = 0
    for w in range(1, maxbits + 1):
        start[w] = acc
        acc += rank[w] << (w - 1)
    size = 1 << maxbits
    tsym = [0] * size
    tbits = [0] * size
    for s, w in enumerate(weights):
        if not w:
            continue
        ln = 1 << (w - 1)
        b = maxbits + 1 - w
        for u in range(start[w], start[w] + ln):
            tsym[u] = s
            tbits[u] = b
        start[w] += ln
    return (tsym, tbits, maxbits), used_total


def _huffman_stream(data, table, n):
    tsym, tbits, maxbits = table
    br = _BackBits(data)
    out = bytearray(n)
    for i in range(n):
        v = br.peek(maxbits)
        out[i] = tsym[v]
        br.pos -= tbits[v]
    if br.pos != 0:
        raise ZstdError('Huffman stream not consumed exactly')
    return out


def _literals(src, pos, st):
    b0 = src[pos]
    ltype, sf = b0 & 3, (b0 >> 2) & 3
    if ltype < 2:
        if sf in (0, 2):
            regen, h = b0 >> 3, 1
        elif sf == 1:
            regen, h = (b0 >> 4) + (src[pos + 1] << 4), 2
        else:
            regen, h = (b0 >> 4) + (src[pos + 1] << 4) + (src[pos + 2] << 12), 3
        pos += h
        if ltype == 0:
            return bytes(src[pos:pos + regen]), pos + regen
        return bytes([src[pos]]) * regen, pos + 1
    if sf < 2:
        hv = int.from_bytes(src[pos:pos + 3], 'little')
        regen, csize, h, nstreams = (hv >> 4) & 0x3FF, (hv >> 14) & 0x3FF, 3, 1 if sf == 0 else 4
    elif sf == 2:
        hv = int.from_bytes(src[pos:pos + 4], 'little')
        regen, csize, h, nstreams = (hv >> 4) & 0x3FFF, (hv >> 18) & 0x3FFF, 4, 4
    else:
        hv = int.from_bytes(src[pos:pos + 5], 'little')
        regen, csize, h, nstreams = (hv >> 4) & 0x3FFFF, (hv >> 22) & 0x3FFFF, 5, 4
    pos += h
    end = pos + csize
    if ltype == 2:
        st['huf'], used = _huffman_table(src, pos)
        pos += used
    elif st.get('huf') is None:
        raise ZstdError('treeless literals without a previous Huffman table')
    table = st['huf']
    if nstreams == 1:
        return bytes(_huffman_stream(src[pos:end], table, regen)), end
    s1, s2, s3 = (int.from_bytes(src[pos + 2 * i:pos + 2 * i + 2], 'little') for i in range(3))
    pos += 6
    q = (regen + 3) // 4
    sizes = [s1, s2, s3, end - pos - s1 - s2 - s3]
    if sizes[3] < 0:
        raise ZstdError('Huffman jump table beyond the literals section')
    out = bytearray()
    for k in range(4):
        out += _huffman_stream(src[pos:pos + sizes[k]], table, q if k < 3 else regen - 3 * q)
        pos += sizes[k]
    return bytes(out), end


# ---- sequences (RFC 8878 3.1.1.3.2) ----------------------------------------------
def _seq_table(src, pos, mode, which, st, max_sym, max_log):
    if mode == 0:
        t = _default_table(which)
    elif mode == 1:
        t = ([src[pos]], [0], [0], 0)
        pos += 1
    elif mode == 2:
        counts, acc, used = _read_distribution(src, pos, max_sym, max_log)
        t = _fse_table(counts, acc)
        pos += used
    else:
        t = st.get(which)
        if t is None:
            raise ZstdError('repeat mode without a previous table')
    st[which] = t
    return t, pos


def _sequences(src, pos, end, st):
    b0 = src[pos]
    if b0 == 0:
        return [], pos + 1
    if b0 < 128:
        n, pos = b0, pos + 1
    elif b0 < 255:
        n, pos = ((b0 - 128) << 8) + src[pos + 1], pos + 2
    else:
        n, pos = src[pos + 1] + (src[pos + 2] << 8) + 0x7F00, pos + 3
    modes = src[pos]
    pos += 1
    if modes & 3:
        raise ZstdError('reserved bits set in the sequence modes')
    ll_t, pos = _seq_table(src, pos, modes >> 6, 'll', st, 36, 9)
    of_t, pos = _seq_table(src, pos, (modes >> 4) & 3, 'of', st, 32, 8)
    ml_t, pos = _seq_table(src, pos, (modes >> 2) & 3, 'ml', st, 53, 9)
    br = _BackBits(src[pos:end])
    lls, lln, llb, lla = ll_t
    ofs, ofn, ofb, ofa = of_t
    mls, mln, mlb, mla = ml_t
    sl = br.read(lla)
    so = br.read(ofa)
    sm = br.read(mla)
    seqs = []
    for i in range(n):
        oc = ofs[so]
        mc = mls[sm]
        lc = lls[sl]
        if oc > 31 or mc > 52 or lc > 35:
            raise ZstdError('sequence code out of range')
        off = (1 << oc) + br.read(oc)
        ml = _ML_BASE[mc] + br.read(_ML_BITS[mc])
        ll = _LL_BASE[lc] + br.read(_LL_BITS[lc])
        seqs.append((ll, ml, off))
        if i + 1 < n:
            sl = llb[sl] + br.read(lln[sl])
            sm = mlb[sm] + br.read(mln[sm])
            so = ofb[so] + br.read(ofn[so])
    if br.pos != 0:
        raise ZstdError('sequence bit stream not consumed exactly')
    return seqs, end


def _execute(seqs, lits, out, frame_start, st):
    rep = st['rep']
    li = 0
    for ll, ml, ov in seqs:
        if ll:
            out += lits[li:li + ll]
            li += ll
        if ov > 3:
            off = ov - 3
            rep[:] = [off, rep[0], rep[1]]
        else:
            k = ov + (1 if ll == 0 else 0)
            if k == 1:
                off = rep[0]
            elif k == 2:
                off = rep[1]
                rep[:] = [rep[1], rep[0], rep[2]]
            elif k == 3:
                off = rep[2]
                rep[:] = [rep[2], rep[0], rep[1]]
            else:
                off = rep[0] - 1
                rep[:] = [off, rep[0], rep[1]]
        if off <= 0 or off > len(out) - frame_start:
            raise ZstdError('match offset outside the decoded data')
        start = len(out) - off
        if off >= ml:
            out += out[start:start + ml]
        else:   # overlapping copy: the match repeats its last `off` bytes
            chunk = bytes(out[start:])
            reps, r = divmod(ml, off)
            out += chunk * reps + chunk[:r]
    if li > len(lits):
        raise ZstdError('sequences use more literals than decoded')
    out += lits[li:]


# ---- XXH64 (the frame content checksum) -----------------------------------------
_M64 = (1 << 64) - 1
_P1, _P2, _P3, _P4, _P5 = (11400714785074694791, 14029467366897019727, 1609587929392839161, 9650029242287828579,
                           2870177450012600261)


def _rotl(x, r):
    return ((x << r) | (x >> (64 - r))) & _M64


def _round(acc, v):
    return (_rotl((acc + v * _P2) & _M64, 31) * _P1) & _M64


def xxh64(data, seed=0):
    """XXH64 of data (Yann Collet's published algorithm)."""
    n = len(data)
    p = 0
    if n >= 32:
        v1, v2, v3, v4 = (seed + _P1 + _P2) & _M64, (seed + _P2) & _M64, seed, (seed - _P1) & _M64
        lim = n - 32
        mv = memoryview(data)
        while p <= lim:
            a, b, c, d = mv[p:p + 32].cast('Q')
            v1, v2, v3, v4 = _round(v1, a), _round(v2, b), _round(v3, c), _round(v4, d)
            p += 32
        h = (_rotl(v1, 1) + _rotl(v2, 7) + _rotl(v3, 12) + _rotl(v4, 18)) & _M64
        for v in (v1, v2, v3, v4):
            h = ((h ^ _round(0, v)) * _P1 + _P4) & _M64
    else:
        h = (seed + _P5) & _M64
    h = (h + n) & _M64
    while p + 8 <= n:
        h ^= _round(0, int.from_bytes(data[p:p + 8], 'little'))
        h = (_rotl(h, 27) * _P1 + _P4) & _M64
        p += 8
    if p + 4 <= n:
        h ^= (int.from_bytes(data[p:p + 4], 'little') * _P1) & _M64
        h = (_rotl(h, 23) * _P2 + _P3) & _M64
        p += 4
    while p < n:
        h ^= (data[p] * _P5) & _M64
        h = (_rotl(h, 11) * _P1) & _M64
        p += 1
    h ^= h >> 33
    h = (h * _P2) & _M64
    h ^= h >> 29
    h = (h * _P3) & _M64
    h ^= h >> 32
    return h


# ---- frames -------------------------------------------------------------------
def _frame(src, pos, out, verify):
    fhd = src[pos]
    pos += 1
    if fhd & 0x08:
        raise ZstdError('reserved bit set in the frame header')
    fcs_flag, single, has_ck, did_flag = fhd >> 6, (fhd >> 5) & 1, (fhd >> 2) & 1, fhd & 3
    if not single:
        pos += 1   # window descriptor: the whole frame is kept, so its size is not needed
    did_n = (0, 1, 2, 4)[did_flag]
    if did_n and int.from_bytes(src[pos:pos + did_n], 'little') != 0:
        raise ZstdError('zstd dictionaries are not supported')
    pos += did_n
    fcs_n = (1 if single else 0, 2, 4, 8)[fcs_flag]
    fcs = None
    if fcs_n:
        fcs = int.from_bytes(src[pos:pos + fcs_n], 'little') + (256 if fcs_n == 2 else 0)
        pos += fcs_n
    start = len(out)
    st = {'rep': [1, 4, 8]}
    while True:
        if pos + 3 > len(src):
            raise ZstdError('truncated block header')
        bh = int.from_bytes(src[pos:pos + 3], 'little')
        pos += 3
        last, btype, bsize = bh & 1, (bh >> 1) & 3, bh >> 3
        if btype == 0:
            out += src[pos:pos + bsize]
            pos += bsize
        elif btype == 1:
            out += bytes([src[pos]]) * bsize
            pos += 1
        elif btype == 2:
            end = pos + bsize
            lits, p = _literals(src, pos, st)
            seqs, _ = _sequences(src, p, end, st)
            _execute(seqs, lits, out, start, st)
            pos = end
        else:
            raise ZstdError('reserved block type')
        if last:
            break
    if fcs is not None and len(out) - start != fcs:
        raise ZstdError(f'frame content size {fcs}, decoded {len(out) - start}')
    if has_ck:
        ck = int.from_bytes(src[pos:pos + 4], 'little')
        pos += 4
        if verify and (xxh64(bytes(out[start:])) & 0xFFFFFFFF) != ck:
            raise ZstdError('content checksum mismatch')
    return pos


def decompress(data, verify=True):
    """Decompress one or more concatenated zstd frames (skippable frames are
    skipped). verify checks the content checksums the frames carry."""
    src = bytes(data)
    out = bytearray()
    pos = 0
    while pos < len(src):
        if pos + 4 > len(src):
            raise ZstdError('truncated frame')
        magic = int.from_bytes(src[pos:pos + 4], 'little')
        if (magic & 0xFFFFFFF0) == 0x184D2A50:
            pos += 8 + int.from_bytes(src[pos + 4:pos + 8], 'little')
            continue
        if magic != _MAGIC:
            raise ZstdError(f'not a zstd frame (magic {magic:#x})')
        pos = _frame(src, pos + 4, out, verify)
    return bytes(out)
