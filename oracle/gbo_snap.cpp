// gbo_snap.cpp -- CPU oracle of the SNAP layer codec (TEST INFRASTRUCTURE
// ONLY: linked into libgbo_oracle.so, used by tests/ and the CPU legs of
// bench.py as the checker; the product library never calls it).
//
// Restates, per 65536-box chunk:
//   * the box codec of box_codec.f90: CompressBoxesUsingCodec (:616-698) and
//     DecompressBoxesUsingCodec (:446-525), with zigzag_encode/decode
//     (:334-356), write_varint/read_varint (:358-396) and the int16 index
//     (:412-441, little-endian);
//   * the Snappy raw block format that snappy_api.cpp:9-37 wraps
//     (snappy::RawCompress / RawUncompress, a third-party library that the
//     reference does not vendor; its published format: a varint preamble with
//     the uncompressed length, then literal and copy elements with 1-, 2- or
//     4-byte offsets).  The decoder accepts every element of that format.  The
//     compressor is this project's own deterministic greedy parse (below),
//     whose output any Snappy decoder reads; it is not byte-identical to the
//     Snappy library's compressor.
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

namespace {

inline uint64_t zigzag(int32_t v) {  // box_codec.f90:334-349
  const int64_t t = v;
  return t < 0 ? (uint64_t)(-t) * 2u - 1u : (uint64_t)t * 2u;
}
inline int32_t unzigzag(uint64_t v) {  // box_codec.f90:351-356
  return (int32_t)(uint32_t)((v >> 1) ^ (uint64_t)(-(int64_t)(v & 1u)));
}
inline int put_varint(uint8_t* o, uint64_t v) {  // box_codec.f90:358-378
  int n = 0;
  while (v >= 128u) {
    o[n++] = (uint8_t)(v | 128u);
    v >>= 7;
  }
  o[n++] = (uint8_t)v;
  return n;
}
// returns bytes consumed, 0 when the varint runs past len or exceeds 10 bytes
inline int get_varint(const uint8_t* s, int64_t pos, int64_t len, uint64_t* v) {
  uint64_t r = 0;
  for (int i = 0; i < 10; ++i) {
    if (pos + i >= len) return 0;
    const uint8_t b = s[pos + i];
    r |= (uint64_t)(b & 127u) << (7 * i);
    if (!(b & 128u)) {
      *v = r;
      return i + 1;
    }
  }
  return 0;
}

inline uint32_t ld32(const uint8_t* p) {
  uint32_t v;
  std::memcpy(&v, p, 4);
  return v;
}

int emit_literal(uint8_t* o, const uint8_t* src, int64_t len) {
  int n = 0;
  const uint64_t m = (uint64_t)len - 1u;
  if (m < 60) {
    o[n++] = (uint8_t)(m << 2);
  } else {
    int nb = m < 256u ? 1 : m < 65536u ? 2 : m < (1u << 24) ? 3 : 4;
    o[n++] = (uint8_t)((59 + nb) << 2);
    for (int i = 0; i < nb; ++i) o[n++] = (uint8_t)(m >> (8 * i));
  }
  std::memcpy(o + n, src, (size_t)len);
  return n + (int)len;
}

int emit_copy_upto64(uint8_t* o, uint32_t off, int len) {  // 4 <= len <= 64
  if (len <= 11 && off < 2048u) {
    o[0] = (uint8_t)(1u | ((uint32_t)(len - 4) << 2) | ((off >> 8) << 5));
    o[1] = (uint8_t)off;
    return 2;
  }
  o[0] = (uint8_t)(2u | ((uint32_t)(len - 1) << 2));
  o[1] = (uint8_t)off;
  o[2] = (uint8_t)(off >> 8);
  return 3;
}

int emit_copy(uint8_t* o, uint32_t off, int64_t len) {
  int n = 0;
  while (len >= 68) {
    n += emit_copy_upto64(o + n, off, 64);
    len -= 64;
  }
  if (len > 64) {
    n += emit_copy_upto64(o + n, off, 60);
    len -= 60;
  }
  return n + emit_copy_upto64(o + n, off, (int)len);
}

}  // namespace

extern "C" {

// One chunk of boxes (x1,y1,x2,y2 int32) into the codec byte stream; out must
// hold 32 bytes per box.  Returns the bytes written.
int64_t orc_codec_encode(const int32_t* b, int64_t n, uint8_t* out) {
  std::unordered_map<int32_t, int64_t> wi, hi;  // value -> 1-based index of first appearance
  int64_t cur_w = 0, cur_h = 0, nw = 0, nh = 0;
  int32_t cx = 0, cy = 0;
  int64_t pos = 0;
  for (int64_t i = 0; i < n; ++i) {
    const int32_t x1 = b[4 * i], y1 = b[4 * i + 1], x2 = b[4 * i + 2], y2 = b[4 * i + 3];
    const int32_t w = (int32_t)((uint32_t)x2 - (uint32_t)x1), h = (int32_t)((uint32_t)y2 - (uint32_t)y1);
    uint8_t info = 0;
    const bool sq = w == h;
    if (sq) info |= 16;
    const int32_t dx = (int32_t)((uint32_t)x1 - (uint32_t)cx), dy = (int32_t)((uint32_t)y1 - (uint32_t)cy);
    if (dx != 0) {
      info |= 32;
      cx = x1;
    }
    if (dy != 0) {
      info |= 64;
      cy = y1;
    }
    auto fw = wi.find(w);
    int64_t widx = fw == wi.end() ? -1 : fw->second;
    bool wnew = false;
    if (widx != cur_w || nw == 0) {
      info |= 1;
      if (widx <= 0) {
        info |= 2;
        wnew = true;
        widx = ++nw;
        wi[w] = widx;
      }
      cur_w = widx;
    }
    int64_t hidx = 0;
    bool hnew = false;
    if (!sq) {
      auto fh = hi.find(h);
      hidx = fh == hi.end() ? -1 : fh->second;
      if (hidx != cur_h || nh == 0) {
        info |= 4;
        if (hidx <= 0) {
          info |= 8;
          hnew = true;
          hidx = ++nh;
          hi[h] = hidx;
        }
        cur_h = hidx;
      }
    }
    out[pos++] = info;
    if (info & 32) pos += put_varint(out + pos, zigzag(dx));
    if (info & 64) pos += put_varint(out + pos, zigzag(dy));
    if (info & 1) {
      if (wnew) {
        pos += put_varint(out + pos, (uint64_t)(int64_t)w);
      } else {
        const uint16_t wire = (uint16_t)widx;
        out[pos++] = (uint8_t)wire;
        out[pos++] = (uint8_t)(wire >> 8);
      }
    }
    if (!sq && (info & 4)) {
      if (hnew) {
        pos += put_varint(out + pos, (uint64_t)(int64_t)h);
      } else {
        const uint16_t wire = (uint16_t)hidx;
        out[pos++] = (uint8_t)wire;
        out[pos++] = (uint8_t)(wire >> 8);
      }
    }
  }
  return pos;
}

// Decodes n boxes of one chunk.  Returns 0, or -(i+1) when record i reads
// past the stream or names an index the dictionary does not hold (the
// reference stops with "Stream Desync" there).
int64_t orc_codec_decode(const uint8_t* s, int64_t len, int64_t n, int32_t* b) {
  std::vector<int32_t> uw, uh;
  int64_t cur_w = 0, cur_h = 0;
  int32_t cx = 0, cy = 0;
  int64_t pos = 0;
  for (int64_t i = 0; i < n; ++i) {
    if (pos >= len) return -(i + 1);
    const uint8_t info = s[pos++];
    const bool sq = info & 16;
    uint64_t v;
    int k;
    if (info & 32) {
      if (!(k = get_varint(s, pos, len, &v))) return -(i + 1);
      pos += k;
      cx = (int32_t)((uint32_t)cx + (uint32_t)unzigzag(v));
    }
    if (info & 64) {
      if (!(k = get_varint(s, pos, len, &v))) return -(i + 1);
      pos += k;
      cy = (int32_t)((uint32_t)cy + (uint32_t)unzigzag(v));
    }
    int32_t w, h;
    if (info & 1) {
      if (info & 2) {
        if (!(k = get_varint(s, pos, len, &v))) return -(i + 1);
        pos += k;
        w = (int32_t)(uint32_t)v;
        uw.push_back(w);
        cur_w = (int64_t)uw.size();
      } else {
        if (pos + 2 > len) return -(i + 1);
        const int16_t wire = (int16_t)(uint16_t)(s[pos] | (s[pos + 1] << 8));
        pos += 2;
        if (wire < 1 || wire > (int64_t)uw.size()) return -(i + 1);
        w = uw[wire - 1];
        cur_w = wire;
      }
    } else {
      if (cur_w < 1) return -(i + 1);
      w = uw[cur_w - 1];
    }
    if (sq) {
      h = w;
    } else if (info & 4) {
      if (info & 8) {
        if (!(k = get_varint(s, pos, len, &v))) return -(i + 1);
        pos += k;
        h = (int32_t)(uint32_t)v;
        uh.push_back(h);
        cur_h = (int64_t)uh.size();
      } else {
        if (pos + 2 > len) return -(i + 1);
        const int16_t wire = (int16_t)(uint16_t)(s[pos] | (s[pos + 1] << 8));
        pos += 2;
        if (wire < 1 || wire > (int64_t)uh.size()) return -(i + 1);
        h = uh[wire - 1];
        cur_h = wire;
      }
    } else {
      if (cur_h < 1) return -(i + 1);
      h = uh[cur_h - 1];
    }
    b[4 * i] = cx;
    b[4 * i + 1] = cy;
    b[4 * i + 2] = (int32_t)((uint32_t)cx + (uint32_t)w);
    b[4 * i + 3] = (int32_t)((uint32_t)cy + (uint32_t)h);
  }
  return 0;
}

// Upper bound of orc_snappy_compress's output for len input bytes.
int64_t orc_snappy_max_length(int64_t len) { return 32 + len + len / 6; }

// Snappy raw format, this project's greedy parse: the input is cut into
// 65536-byte fragments compressed independently (offsets never reach before
// the fragment).  Every position p with 4 bytes left in the fragment has a
// candidate: the latest earlier position whose 4 bytes hash to the same slot
// ((v * 0x9E3779B1) >> 21, Knuth's multiplicative hash into 2048 slots;
// every position is hashed, including those inside matches).  The parse
// starts at 0; at p, when the candidate's 4 bytes equal those at p, the match
// is extended as far as the fragment allows and, when at least 8 bytes long,
// emitted (pending literal first) and p jumps past it; otherwise p advances
// by one.  (Shorter matches save at most a few bytes but add elements, which
// a decoder has to take one after another.)  Copies are split
// into pieces of 64 (60 when 65..67 remain), each piece a 1-byte-offset copy
// when 4..11 long with offset < 2048, else a 2-byte-offset copy.
int64_t orc_snappy_compress(const uint8_t* in, int64_t len, uint8_t* out) {
  int64_t o = put_varint(out, (uint64_t)len);
  std::vector<uint32_t> table(2048), cand(65536);
  for (int64_t f0 = 0; f0 < len; f0 += 65536) {
    const int64_t fl = len - f0 < 65536 ? len - f0 : 65536;
    const uint8_t* s = in + f0;
    std::fill(table.begin(), table.end(), 0u);
    for (int64_t p = 0; p + 4 <= fl; ++p) {  // candidate of every position (1-based, 0 = none)
      const uint32_t h = (ld32(s + p) * 0x9E3779B1u) >> 21;
      cand[p] = table[h];
      table[h] = (uint32_t)p + 1u;
    }
    int64_t p = 0, lit = 0;
    while (p + 4 <= fl) {
      const uint32_t c = cand[p];
      if (c && ld32(s + c - 1) == ld32(s + p)) {
        const int64_t q = c - 1;
        int64_t L = 4;
        while (p + L < fl && s[q + L] == s[p + L]) ++L;
        if (L >= 8) {
          if (p > lit) o += emit_literal(out + o, s + lit, p - lit);
          o += emit_copy(out + o, (uint32_t)(p - q), L);
          p += L;
          lit = p;
          continue;
        }
      }
      ++p;
    }
    if (fl > lit) o += emit_literal(out + o, s + lit, fl - lit);
  }
  return o;
}

// Uncompressed length from the preamble, or -1.
int64_t orc_snappy_uncompressed_length(const uint8_t* in, int64_t len) {
  uint64_t v;
  const int k = get_varint(in, 0, len < 5 ? len : 5, &v);
  if (!k || v > 0xFFFFFFFFull) return -1;
  return (int64_t)v;
}

// Decodes any Snappy raw stream into out (cap bytes).  Returns the bytes
// produced, or -1 for a malformed stream (offset 0 or before the output
// start, element past the input, output past cap or short of the preamble).
int64_t orc_snappy_decompress(const uint8_t* in, int64_t len, uint8_t* out, int64_t cap) {
  uint64_t want;
  int64_t p = get_varint(in, 0, len < 5 ? len : 5, &want);
  if (!p || (int64_t)want > cap) return -1;
  int64_t o = 0;
  while (p < len) {
    const uint8_t tag = in[p++];
    const int t = tag & 3;
    if (t == 0) {
      int64_t m = tag >> 2;
      if (m >= 60) {
        const int nb = (int)m - 59;
        if (p + nb > len) return -1;
        m = 0;
        for (int i = 0; i < nb; ++i) m |= (int64_t)in[p + i] << (8 * i);
        p += nb;
      }
      const int64_t L = m + 1;
      if (p + L > len || o + L > (int64_t)want) return -1;
      std::memcpy(out + o, in + p, (size_t)L);
      p += L;
      o += L;
      continue;
    }
    int64_t L, off;
    if (t == 1) {
      if (p + 1 > len) return -1;
      L = 4 + ((tag >> 2) & 7);
      off = ((int64_t)(tag >> 5) << 8) | in[p];
      p += 1;
    } else if (t == 2) {
      if (p + 2 > len) return -1;
      L = 1 + (tag >> 2);
      off = in[p] | ((int64_t)in[p + 1] << 8);
      p += 2;
    } else {
      if (p + 4 > len) return -1;
      L = 1 + (tag >> 2);
      off = (int64_t)in[p] | ((int64_t)in[p + 1] << 8) | ((int64_t)in[p + 2] << 16) | ((int64_t)in[p + 3] << 24);
      p += 4;
    }
    if (off == 0 || off > o || o + L > (int64_t)want) return -1;
    for (int64_t i = 0; i < L; ++i) out[o + i] = out[o + i - off];  // overlapping copies repeat the pattern
    o += L;
  }
  return o == (int64_t)want ? o : -1;
}

}  // extern "C"
