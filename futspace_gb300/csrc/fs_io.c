/*
 * Map ingest and frame output on the host: PNG images and the Futhark binary
 * data format, the two on-disk forms the reference's tools and front end use.
 *
 *  - PNG read (c/freeimage_futspace.h:19-58 loads map images through FreeImage
 *    into 0xFF000000 | R << 16 | G << 8 | B words, rows top to bottom): 8-bit
 *    greyscale, RGB, palette, grey+alpha and RGBA images without interlacing
 *    (the forms under data/), alpha dropped as FreeImage's loader drops it.
 *    The zlib stream is inflated here (RFC 1950/1951: stored, fixed and dynamic
 *    Huffman blocks, Adler-32 checked); chunk CRCs are checked.
 *  - PNG write: 8-bit RGB, stored deflate blocks (a headless frame dump; the
 *    reference saves screenshots through FreeImage, c/freeimage_futspace.h:60-).
 *  - Futhark binary data format (tools/png2data.py:46-53 writes it,
 *    tools/data2png.py:19-58 reads it): 'b', version 2, rank, a 4-character
 *    element type (" i32", " u32", "  u8", ...), rank little-endian u64
 *    dimensions, then the elements little-endian.
 */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fs_internal.h"
#include "fs_priv.h"

/* ---- inflate (RFC 1951) ----------------------------------------------------- */

typedef struct {
  const uint8_t *in;
  size_t n, pos; /* input bytes, next byte */
  uint32_t buf;  /* bit buffer, least significant bit first */
  int cnt;       /* bits in buf */
  int err;
} bitrd;

static uint32_t bits(bitrd *b, int need) {
  while (b->cnt < need) {
    if (b->pos >= b->n) {
      b->err = 1;
      return 0;
    }
    b->buf |= (uint32_t)b->in[b->pos++] << b->cnt;
    b->cnt += 8;
  }
  const uint32_t v = b->buf & ((need == 32) ? 0xFFFFFFFFu : ((1u << need) - 1u));
  b->buf = need == 32 ? 0 : b->buf >> need;
  b->cnt -= need;
  return v;
}

/* Canonical Huffman code: codes of each length are consecutive, shorter codes
 * first, and symbols of equal length in increasing order. */
typedef struct {
  uint16_t count[16];  /* codes per length */
  uint16_t symbol[320]; /* symbols ordered by (length, value) */
} huff;

static int huff_build(huff *h, const uint8_t *len, int n) {
  memset(h->count, 0, sizeof(h->count));
  for (int s = 0; s < n; s++) h->count[len[s]]++;
  h->count[0] = 0;
  int left = 1; /* over-subscription check */
  for (int l = 1; l < 16; l++) {
    left <<= 1;
    left -= h->count[l];
    if (left < 0) return -1;
  }
  uint16_t offs[16];
  offs[1] = 0;
  for (int l = 1; l < 15; l++) offs[l + 1] = (uint16_t)(offs[l] + h->count[l]);
  for (int s = 0; s < n; s++)
    if (len[s]) h->symbol[offs[len[s]]++] = (uint16_t)s;
  return 0;
}

static int huff_decode(bitrd *b, const huff *h) {
  int code = 0, first = 0, index = 0;
  for (int l = 1; l < 16; l++) {
    code |= (int)bits(b, 1);
    if (b->err) return -1;
    const int c = h->count[l];
    if (code - first < c) return h->symbol[index + (code - first)];
    index += c;
    first = (first + c) << 1;
    code <<= 1;
  }
  return -1; /* no code of any length matched */
}

/* Base values and extra bits of length codes 257..285 and distance codes 0..29
 * (RFC 1951 section 3.2.5). */
static const uint16_t k_len_base[29] = {3,  4,  5,  6,  7,  8,  9,  10, 11,  13,  15,  17,  19,  23, 27,
                                        31, 35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
static const uint8_t k_len_extra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2,
                                        2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
static const uint16_t k_dist_base[30] = {1,    2,    3,    4,    5,    7,     9,     13,    17,  25,
                                         33,   49,   65,   97,   129,  193,   257,   385,   513, 769,
                                         1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
static const uint8_t k_dist_extra[30] = {0, 0, 0, 0, 1, 1, 2, 2,  3,  3,  4,  4,  5,  5,  6,
                                         6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

typedef struct {
  uint8_t *out;
  size_t cap, len;
} outbuf;

static int inflate_codes(bitrd *b, outbuf *o, const huff *lit, const huff *dist) {
  for (;;) {
    int sym = huff_decode(b, lit);
    if (sym < 0) return -1;
    if (sym < 256) {
      if (o->len >= o->cap) return -2;
      o->out[o->len++] = (uint8_t)sym;
    } else if (sym == 256) {
      return 0;
    } else {
      sym -= 257;
      if (sym >= 29) return -1;
      const size_t len = k_len_base[sym] + bits(b, k_len_extra[sym]);
      const int ds = huff_decode(b, dist);
      if (ds < 0 || ds >= 30 || b->err) return -1;
      const size_t d = k_dist_base[ds] + bits(b, k_dist_extra[ds]);
      if (b->err || d > o->len) return -1;
      if (o->len + len > o->cap) return -2;
      for (size_t i = 0; i < len; i++, o->len++) o->out[o->len] = o->out[o->len - d];
    }
  }
}

static int inflate_raw(bitrd *b, outbuf *o) {
  huff lit, dist;
  int last;
  do {
    last = (int)bits(b, 1);
    const int type = (int)bits(b, 2);
    if (b->err) return -1;
    if (type == 0) { /* stored */
      b->buf = 0;
      b->cnt = 0; /* drop to the byte boundary */
      if (b->pos + 4 > b->n) return -1;
      const unsigned len = b->in[b->pos] | (b->in[b->pos + 1] << 8);
      const unsigned nlen = b->in[b->pos + 2] | (b->in[b->pos + 3] << 8);
      b->pos += 4;
      if ((len ^ 0xFFFFu) != nlen || b->pos + len > b->n) return -1;
      if (o->len + len > o->cap) return -2;
      memcpy(o->out + o->len, b->in + b->pos, len);
      o->len += len;
      b->pos += len;
    } else if (type == 1) { /* fixed Huffman codes */
      uint8_t l[320];
      int s = 0;
      for (; s < 144; s++) l[s] = 8;
      for (; s < 256; s++) l[s] = 9;
      for (; s < 280; s++) l[s] = 7;
      for (; s < 288; s++) l[s] = 8;
      huff_build(&lit, l, 288);
      for (s = 0; s < 30; s++) l[s] = 5;
      huff_build(&dist, l, 30);
      const int rc = inflate_codes(b, o, &lit, &dist);
      if (rc) return rc;
    } else if (type == 2) { /* dynamic Huffman codes */
      const int nlen = (int)bits(b, 5) + 257, ndist = (int)bits(b, 5) + 1;
      const int ncode = (int)bits(b, 4) + 4;
      if (b->err || nlen > 286 || ndist > 30) return -1;
      static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5,
                                        11, 4,  12, 3, 13, 2, 14, 1, 15};
      uint8_t cl[19] = {0};
      for (int i = 0; i < ncode; i++) cl[order[i]] = (uint8_t)bits(b, 3);
      huff clh;
      if (b->err || huff_build(&clh, cl, 19)) return -1;
      uint8_t l[320];
      int i = 0;
      while (i < nlen + ndist) {
        int sym = huff_decode(b, &clh);
        if (sym < 0) return -1;
        if (sym < 16) {
          l[i++] = (uint8_t)sym;
        } else {
          int rep, val = 0;
          if (sym == 16) {
            if (i == 0) return -1;
            val = l[i - 1];
            rep = 3 + (int)bits(b, 2);
          } else if (sym == 17) {
            rep = 3 + (int)bits(b, 3);
          } else {
            rep = 11 + (int)bits(b, 7);
          }
          if (b->err || i + rep > nlen + ndist) return -1;
          while (rep--) l[i++] = (uint8_t)val;
        }
      }
      if (l[256] == 0) return -1; /* no end-of-block code */
      if (huff_build(&lit, l, nlen) || huff_build(&dist, l + nlen, ndist)) return -1;
      const int rc = inflate_codes(b, o, &lit, &dist);
      if (rc) return rc;
    } else {
      return -1;
    }
  } while (!last);
  return 0;
}

static uint32_t adler32(const uint8_t *p, size_t n) {
  uint32_t a = 1, s = 0;
  for (size_t i = 0; i < n; i++) {
    a = (a + p[i]) % 65521u;
    s = (s + a) % 65521u;
  }
  return (s << 16) | a;
}

/* zlib stream (RFC 1950) into exactly `cap` bytes. */
static int zlib_inflate(const uint8_t *in, size_t n, uint8_t *out, size_t cap) {
  if (n < 6) return -1;
  const unsigned cmf = in[0], flg = in[1];
  if ((cmf & 15) != 8 || ((cmf << 8) | flg) % 31 != 0 || (flg & 0x20)) return -1;
  bitrd b = {in + 2, n - 2, 0, 0, 0, 0};
  outbuf o = {out, cap, 0};
  const int rc = inflate_raw(&b, &o);
  if (rc) return rc;
  if (o.len != cap || b.pos + 4 > b.n) return -1;
  const uint32_t want = ((uint32_t)b.in[b.pos] << 24) | ((uint32_t)b.in[b.pos + 1] << 16) |
                        ((uint32_t)b.in[b.pos + 2] << 8) | b.in[b.pos + 3];
  return want == adler32(out, cap) ? 0 : -1;
}

/* ---- PNG -------------------------------------------------------------------- */

static uint32_t k_crc[256];
static int k_crc_ready;

static uint32_t crc32_png(const uint8_t *p, size_t n, uint32_t c) {
  if (!k_crc_ready) { /* polynomial 0xEDB88320, reflected */
    for (uint32_t i = 0; i < 256; i++) {
      uint32_t v = i;
      for (int k = 0; k < 8; k++) v = (v & 1) ? 0xEDB88320u ^ (v >> 1) : v >> 1;
      k_crc[i] = v;
    }
    k_crc_ready = 1;
  }
  c = ~c;
  for (size_t i = 0; i < n; i++) c = k_crc[(c ^ p[i]) & 0xFF] ^ (c >> 8);
  return ~c;
}

static uint32_t be32(const uint8_t *p) {
  return ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | p[3];
}

static int read_file(const char *path, uint8_t **data, size_t *n) {
  FILE *f = fopen(path, "rb");
  if (!f) return FS_ERR_IO;
  if (fseek(f, 0, SEEK_END) != 0) {
    fclose(f);
    return FS_ERR_IO;
  }
  const long sz = ftell(f);
  if (sz < 0 || fseek(f, 0, SEEK_SET) != 0) {
    fclose(f);
    return FS_ERR_IO;
  }
  uint8_t *buf = (uint8_t *)malloc((size_t)sz + 1);
  if (!buf) {
    fclose(f);
    return FS_ERR_NOMEM;
  }
  const size_t got = fread(buf, 1, (size_t)sz, f);
  fclose(f);
  if (got != (size_t)sz) {
    free(buf);
    return FS_ERR_IO;
  }
  *data = buf;
  *n = (size_t)sz;
  return FS_OK;
}

static int paeth(int a, int b, int c) {
  const int p = a + b - c;
  const int pa = abs(p - a), pb = abs(p - b), pc = abs(p - c);
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

int fs_png_decode(const uint8_t *png, size_t n, uint32_t **argb, int64_t *rows, int64_t *cols) {
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  if (!png || !argb || !rows || !cols) return FS_ERR_ARG;
  if (n < 8 || memcmp(png, sig, 8) != 0) return FS_ERR_IO;
  uint32_t W = 0, H = 0;
  int depth = 0, ctype = -1, interlace = 0;
  uint8_t pal[256][3];
  int npal = 0;
  uint8_t *idat = NULL;
  size_t idat_n = 0, idat_cap = 0;
  int rc = FS_ERR_IO, seen_end = 0;
  size_t pos = 8;
  while (pos + 12 <= n) {
    const uint32_t len = be32(png + pos);
    const uint8_t *type = png + pos + 4;
    if (len > n - pos - 12) goto done;
    const uint8_t *body = png + pos + 8;
    if (crc32_png(type, (size_t)len + 4, 0) != be32(body + len)) goto done;
    if (!memcmp(type, "IHDR", 4)) {
      if (len != 13) goto done;
      W = be32(body);
      H = be32(body + 4);
      depth = body[8];
      ctype = body[9];
      interlace = body[12];
      if (body[10] != 0 || body[11] != 0) goto done; /* compression, filter method */
    } else if (!memcmp(type, "PLTE", 4)) {
      if (len % 3 || len > 768) goto done;
      npal = (int)(len / 3);
      memcpy(pal, body, len);
    } else if (!memcmp(type, "IDAT", 4)) {
      if (idat_n + len > idat_cap) {
        size_t cap = idat_cap ? idat_cap * 2 : 1 << 20;
        while (cap < idat_n + len) cap *= 2;
        uint8_t *p = (uint8_t *)realloc(idat, cap);
        if (!p) {
          rc = FS_ERR_NOMEM;
          goto done;
        }
        idat = p;
        idat_cap = cap;
      }
      memcpy(idat + idat_n, body, len);
      idat_n += len;
    } else if (!memcmp(type, "IEND", 4)) {
      seen_end = 1;
      break;
    }
    pos += (size_t)len + 12;
  }
  if (!seen_end || W == 0 || H == 0 || W > 65536 || H > 65536) goto done;
  /* 8-bit channels, no interlacing: the forms the reference's maps use */
  int chans;
  switch (ctype) {
    case 0: chans = 1; break;
    case 2: chans = 3; break;
    case 3: chans = 1; break;
    case 4: chans = 2; break;
    case 6: chans = 4; break;
    default: goto done;
  }
  if (depth != 8 || interlace != 0 || (ctype == 3 && npal == 0)) goto done;
  {
    const size_t stride = (size_t)W * chans;
    const size_t raw_n = (stride + 1) * H;
    uint8_t *raw = (uint8_t *)malloc(raw_n);
    uint32_t *img = (uint32_t *)malloc((size_t)W * H * 4);
    if (!raw || !img) {
      free(raw);
      free(img);
      rc = FS_ERR_NOMEM;
      goto done;
    }
    if (!idat || zlib_inflate(idat, idat_n, raw, raw_n) != 0) {
      free(raw);
      free(img);
      goto done;
    }
    /* undo the per-row filters in place (PNG specification, section 9) */
    for (uint32_t y = 0; y < H; y++) {
      uint8_t *row = raw + y * (stride + 1);
      const uint8_t *prev = y ? raw + (y - 1) * (stride + 1) + 1 : NULL;
      const int ft = row[0];
      uint8_t *r = row + 1;
      for (size_t i = 0; i < stride; i++) {
        const int a = i >= (size_t)chans ? r[i - chans] : 0;
        const int b = prev ? prev[i] : 0;
        const int c = (prev && i >= (size_t)chans) ? prev[i - chans] : 0;
        int v;
        switch (ft) {
          case 0: v = 0; break;
          case 1: v = a; break;
          case 2: v = b; break;
          case 3: v = (a + b) >> 1; break;
          case 4: v = paeth(a, b, c); break;
          default: v = -1; break;
        }
        if (v < 0) {
          free(raw);
          free(img);
          goto done;
        }
        r[i] = (uint8_t)(r[i] + v);
      }
      uint32_t *o = img + (size_t)y * W;
      for (uint32_t x = 0; x < W; x++) {
        const uint8_t *px = r + (size_t)x * chans;
        uint32_t R, G, B;
        if (ctype == 0 || ctype == 4) {
          R = G = B = px[0];
        } else if (ctype == 3) {
          if (px[0] >= npal) {
            free(raw);
            free(img);
            goto done;
          }
          R = pal[px[0]][0];
          G = pal[px[0]][1];
          B = pal[px[0]][2];
        } else {
          R = px[0];
          G = px[1];
          B = px[2];
        }
        o[x] = 0xFF000000u | (R << 16) | (G << 8) | B;
      }
    }
    free(raw);
    *argb = img;
    *rows = H;
    *cols = W;
    rc = FS_OK;
  }
done:
  free(idat);
  return rc;
}

int fs_png_read(const char *path, uint32_t **argb, int64_t *rows, int64_t *cols) {
  if (!path || !argb || !rows || !cols) return FS_ERR_ARG;
  uint8_t *data = NULL;
  size_t n = 0;
  int rc = read_file(path, &data, &n);
  if (rc) return rc;
  rc = fs_png_decode(data, n, argb, rows, cols);
  free(data);
  return rc;
}

static void put32(uint8_t *p, uint32_t v) {
  p[0] = (uint8_t)(v >> 24);
  p[1] = (uint8_t)(v >> 16);
  p[2] = (uint8_t)(v >> 8);
  p[3] = (uint8_t)v;
}

static int write_chunk(FILE *f, const char *type, const uint8_t *body, uint32_t len) {
  uint8_t hdr[8];
  put32(hdr, len);
  memcpy(hdr + 4, type, 4);
  uint32_t crc = crc32_png(hdr + 4, 4, 0);
  crc = crc32_png(body, len, crc);
  uint8_t tail[4];
  put32(tail, crc);
  return fwrite(hdr, 1, 8, f) == 8 && (len == 0 || fwrite(body, 1, len, f) == len) &&
                 fwrite(tail, 1, 4, f) == 4
             ? 0
             : -1;
}

int fs_png_write(const char *path, const uint32_t *argb, int64_t rows, int64_t cols) {
  if (!path || !argb || rows <= 0 || cols <= 0 || rows > 65536 || cols > 65536)
    return FS_ERR_ARG;
  const size_t stride = (size_t)cols * 3 + 1;
  const size_t raw_n = stride * (size_t)rows;
  const size_t nblocks = (raw_n + 65534) / 65535;
  const size_t z_n = 2 + raw_n + 5 * nblocks + 4;
  uint8_t *raw = (uint8_t *)malloc(raw_n);
  uint8_t *z = (uint8_t *)malloc(z_n);
  if (!raw || !z) {
    free(raw);
    free(z);
    return FS_ERR_NOMEM;
  }
  for (int64_t y = 0; y < rows; y++) {
    uint8_t *r = raw + (size_t)y * stride;
    r[0] = 0; /* filter: none */
    for (int64_t x = 0; x < cols; x++) {
      const uint32_t c = argb[(size_t)y * (size_t)cols + (size_t)x];
      r[1 + 3 * x] = (uint8_t)(c >> 16);
      r[2 + 3 * x] = (uint8_t)(c >> 8);
      r[3 + 3 * x] = (uint8_t)c;
    }
  }
  /* zlib stream of stored deflate blocks */
  size_t zp = 0;
  z[zp++] = 0x78;
  z[zp++] = 0x01;
  for (size_t off = 0; off < raw_n; off += 65535) {
    const size_t len = raw_n - off < 65535 ? raw_n - off : 65535;
    z[zp++] = (off + len == raw_n) ? 1 : 0;
    z[zp++] = (uint8_t)len;
    z[zp++] = (uint8_t)(len >> 8);
    z[zp++] = (uint8_t)~len;
    z[zp++] = (uint8_t)(~len >> 8);
    memcpy(z + zp, raw + off, len);
    zp += len;
  }
  put32(z + zp, adler32(raw, raw_n));
  zp += 4;
  free(raw);
  FILE *f = fopen(path, "wb");
  if (!f) {
    free(z);
    return FS_ERR_IO;
  }
  static const uint8_t sig[8] = {0x89, 'P', 'N', 'G', '\r', '\n', 0x1A, '\n'};
  uint8_t ihdr[13];
  put32(ihdr, (uint32_t)cols);
  put32(ihdr + 4, (uint32_t)rows);
  ihdr[8] = 8;  /* bit depth */
  ihdr[9] = 2;  /* RGB */
  ihdr[10] = 0; /* deflate */
  ihdr[11] = 0; /* adaptive filtering */
  ihdr[12] = 0; /* no interlace */
  int bad = fwrite(sig, 1, 8, f) != 8;
  bad |= write_chunk(f, "IHDR", ihdr, 13);
  for (size_t off = 0; !bad && off < zp; off += 1u << 20) {
    const size_t len = zp - off < (1u << 20) ? zp - off : (1u << 20);
    bad |= write_chunk(f, "IDAT", z + off, (uint32_t)len);
  }
  bad |= write_chunk(f, "IEND", NULL, 0);
  bad |= fclose(f) != 0;
  free(z);
  return bad ? FS_ERR_IO : FS_OK;
}

/* ---- Futhark binary data format --------------------------------------------- */

static int elem_size(const char type[4]) {
  static const struct {
    const char *name;
    int size;
  } k[] = {{"  i8", 1}, {"  u8", 1}, {" i16", 2}, {" u16", 2}, {" i32", 4}, {" u32", 4},
           {" f32", 4}, {" i64", 8}, {" u64", 8}, {" f64", 8}, {"bool", 1}};
  for (size_t i = 0; i < sizeof(k) / sizeof(k[0]); i++)
    if (!memcmp(type, k[i].name, 4)) return k[i].size;
  return 0;
}

int fs_data_write(const char *path, const void *data, const char *type, int32_t rank,
                  const int64_t *dims) {
  if (!path || !type || rank < 0 || rank > 8 || (rank && !dims) || strlen(type) != 4)
    return FS_ERR_ARG;
  const int es = elem_size(type);
  if (!es) return FS_ERR_ARG;
  uint64_t count = 1;
  for (int i = 0; i < rank; i++) {
    if (dims[i] < 0) return FS_ERR_ARG;
    count *= (uint64_t)dims[i];
  }
  if (count && !data) return FS_ERR_ARG;
  FILE *f = fopen(path, "wb");
  if (!f) return FS_ERR_IO;
  uint8_t hdr[7 + 8 * 8];
  size_t hp = 0;
  hdr[hp++] = 'b';
  hdr[hp++] = 2;
  hdr[hp++] = (uint8_t)rank;
  memcpy(hdr + hp, type, 4);
  hp += 4;
  for (int i = 0; i < rank; i++)
    for (int k = 0; k < 8; k++) hdr[hp++] = (uint8_t)((uint64_t)dims[i] >> (8 * k));
  int bad = fwrite(hdr, 1, hp, f) != hp;
  /* elements little-endian, written byte by byte so the host's order does not
   * matter */
  const uint8_t *p = (const uint8_t *)data;
  uint8_t buf[8192];
  size_t bp = 0;
  const uint16_t one = 1;
  const int little = *(const uint8_t *)&one == 1;
  for (uint64_t i = 0; !bad && i < count; i++) {
    for (int k = 0; k < es; k++) buf[bp++] = p[i * es + (little ? k : es - 1 - k)];
    if (bp + 8 > sizeof(buf)) {
      bad |= fwrite(buf, 1, bp, f) != bp;
      bp = 0;
    }
  }
  if (!bad && bp) bad |= fwrite(buf, 1, bp, f) != bp;
  bad |= fclose(f) != 0;
  return bad ? FS_ERR_IO : FS_OK;
}

int fs_data_read(const char *path, void **data, char type[5], int32_t *rank, int64_t dims[8]) {
  if (!path || !data || !type || !rank || !dims) return FS_ERR_ARG;
  uint8_t *buf = NULL;
  size_t n = 0;
  int rc = read_file(path, &buf, &n);
  if (rc) return rc;
  rc = FS_ERR_IO;
  if (n < 7 || buf[0] != 'b' || buf[1] != 2 || buf[2] > 8) goto done;
  {
    const int r = buf[2];
    memcpy(type, buf + 3, 4);
    type[4] = 0;
    const int es = elem_size(type);
    if (!es || n < 7 + 8 * (size_t)r) goto done;
    uint64_t count = 1;
    for (int i = 0; i < r; i++) {
      uint64_t d = 0;
      for (int k = 0; k < 8; k++) d |= (uint64_t)buf[7 + 8 * i + k] << (8 * k);
      if (d > ((uint64_t)1 << 40)) goto done;
      dims[i] = (int64_t)d;
      count *= d;
      if (count > ((uint64_t)1 << 40)) goto done;
    }
    const size_t off = 7 + 8 * (size_t)r;
    if (n - off != count * (uint64_t)es) goto done;
    const size_t bytes = (size_t)count * (size_t)es;
    uint8_t *out = (uint8_t *)malloc(bytes ? bytes : 1);
    if (!out) {
      rc = FS_ERR_NOMEM;
      goto done;
    }
    const uint16_t one = 1;
    const int little = *(const uint8_t *)&one == 1;
    for (uint64_t i = 0; i < count; i++)
      for (int k = 0; k < es; k++) out[i * es + (little ? k : es - 1 - k)] = buf[off + i * es + k];
    *data = out;
    *rank = r;
    rc = FS_OK;
  }
done:
  free(buf);
  return rc;
}

void fs_free(void *p) { free(p); }

/* Both map images as c/interactive.c:43-56 loads them: colours as ARGB words,
 * heights from the low byte of each word (update_map keeps `& 0xFF`). */
int fs_map_load_png(fs_ctx *ctx, fs_map **out, const char *color_png, const char *height_png) {
  if (!ctx || !out || !color_png || !height_png) return fs_fail(ctx, FS_ERR_ARG, "NULL argument");
  uint32_t *c = NULL, *h = NULL;
  int64_t cr = 0, cc = 0, hr = 0, hc = 0;
  int rc = fs_png_read(color_png, &c, &cr, &cc);
  if (rc) return fs_fail(ctx, rc, "cannot read colour map %s", color_png);
  rc = fs_png_read(height_png, &h, &hr, &hc);
  if (rc) {
    free(c);
    return fs_fail(ctx, rc, "cannot read height map %s", height_png);
  }
  if (cr != hr || cc != hc) {
    free(c);
    free(h);
    return fs_fail(ctx, FS_ERR_ARG, "colour map %lldx%lld and height map %lldx%lld differ",
                   (long long)cr, (long long)cc, (long long)hr, (long long)hc);
  }
  rc = fs_map_new_i32(ctx, out, (const int32_t *)h, c, hr, hc);
  free(c);
  free(h);
  return rc;
}
