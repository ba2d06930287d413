/* The LIME record container (c-lime 1.x: the reader and writer calls
 * lib/src/qcd_io.c makes), restated from the published LIME format for the
 * CPU oracle. Test infrastructure only: it lets the reference's own
 * qcd_io.c readers and writers run (oracle/_ref/libqcdio.so); nothing in
 * the product links it.
 *
 * c-lime itself is not in the reference tree (only its headers are
 * vendored, include/lime*.h). Its format: every record is a 144-byte
 * header -- the magic number 0x456789ab (4 bytes), the version 1
 * (2 bytes), the message-begin / message-end flags in bits 15 / 14 of the
 * next 2 bytes, the payload length (8 bytes), all big-endian, then the
 * NUL-padded record type (128 bytes) -- followed by the payload, padded
 * with zero bytes to a multiple of 8.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <lime.h>

enum { HDR = 144, TYPE_LEN = 128 };

static uint64_t be_get(const unsigned char *p, int n)
{
  uint64_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}

static void be_put(unsigned char *p, uint64_t v, int n)
{
  for (int i = n - 1; i >= 0; i--) {
    p[i] = (unsigned char)(v & 0xff);
    v >>= 8;
  }
}

static size_t pad8(n_uint64_t n) { return (size_t)((8 - n % 8) % 8); }

LimeRecordHeader *limeCreateHeader(int MB_flag, int ME_flag, char *type, n_uint64_t reclen)
{
  if (!type || strlen(type) >= TYPE_LEN) return NULL;
  LimeRecordHeader *h = calloc(1, sizeof(*h));
  if (!h) return NULL;
  h->lime_version = LIME_VERSION;
  h->MB_flag = MB_flag;
  h->ME_flag = ME_flag;
  h->type = malloc(strlen(type) + 1);
  if (!h->type) {
    free(h);
    return NULL;
  }
  strcpy(h->type, type);
  h->data_length = reclen;
  return h;
}

void limeDestroyHeader(LimeRecordHeader *h)
{
  if (!h) return;
  free(h->type);
  free(h);
}

/* ---------------------------------------------------------------- reader */
LimeReader *limeCreateReader(FILE *fp)
{
  if (!fp) return NULL;
  LimeReader *r = calloc(1, sizeof(*r));
  if (!r) return NULL;
  r->fp = fp;
  r->first_read = 1;
  r->header_nextP = 1;
  return r;
}

void limeDestroyReader(LimeReader *r)
{
  if (!r) return;
  limeDestroyHeader(r->curr_header);
  free(r);
}

int limeReaderNextRecord(LimeReader *r)
{
  if (!r) return LIME_ERR_PARAM;
  if (r->curr_header) {  // skip what is left of the current record and its padding
    if (fseeko(r->fp, (off_t)(r->rec_start + r->bytes_total + r->bytes_pad), SEEK_SET)) return LIME_ERR_SEEK;
    limeDestroyHeader(r->curr_header);
    r->curr_header = NULL;
  }
  unsigned char h[HDR];
  size_t got = fread(h, 1, HDR, r->fp);
  if (got == 0) return LIME_EOF;
  if (got != HDR || be_get(h, 4) != LIME_MAGIC_NO) return LIME_ERR_READ;
  char type[TYPE_LEN + 1];
  memcpy(type, h + 16, TYPE_LEN);
  type[TYPE_LEN] = 0;
  const unsigned flags = (unsigned)be_get(h + 6, 2);
  r->curr_header = limeCreateHeader((flags >> 15) & 1, (flags >> 14) & 1, type, be_get(h + 8, 8));
  if (!r->curr_header) return LIME_ERR_READ;
  r->curr_header->lime_version = (unsigned)be_get(h + 4, 2);
  r->first_read = 0;
  r->header_nextP = 0;
  r->is_last = r->curr_header->ME_flag;
  r->bytes_total = r->bytes_left = r->curr_header->data_length;
  r->rec_ptr = 0;
  r->rec_start = (n_uint64_t)ftello(r->fp);
  r->bytes_pad = pad8(r->bytes_total);
  return LIME_SUCCESS;
}

char *limeReaderType(LimeReader *r) { return r && r->curr_header ? r->curr_header->type : NULL; }

n_uint64_t limeReaderBytes(LimeReader *r) { return r ? r->bytes_total : 0; }

int limeReaderReadData(void *dest, n_uint64_t *nbytes, LimeReader *r)
{
  if (!r || !dest || !nbytes || !r->curr_header) return LIME_ERR_PARAM;
  n_uint64_t n = *nbytes < r->bytes_left ? *nbytes : r->bytes_left;
  if (fseeko(r->fp, (off_t)(r->rec_start + r->rec_ptr), SEEK_SET)) return LIME_ERR_SEEK;
  size_t got = fread(dest, 1, (size_t)n, r->fp);
  r->rec_ptr += got;
  r->bytes_left -= got;
  *nbytes = got;
  return got == n ? LIME_SUCCESS : LIME_ERR_READ;
}

/* ---------------------------------------------------------------- writer */
LimeWriter *limeCreateWriter(FILE *fp)
{
  if (!fp) return NULL;
  LimeWriter *w = calloc(1, sizeof(*w));
  if (!w) return NULL;
  w->fp = fp;
  w->first_record = 1;
  w->header_nextP = 1;
  return w;
}

int limeDestroyWriter(LimeWriter *w)
{
  free(w);
  return LIME_SUCCESS;
}

int limeWriteRecordHeader(LimeRecordHeader *props, LimeWriter *w)
{
  if (!props || !w || !props->type) return LIME_ERR_PARAM;
  unsigned char h[HDR];
  memset(h, 0, sizeof(h));
  be_put(h, LIME_MAGIC_NO, 4);
  be_put(h + 4, LIME_VERSION, 2);
  be_put(h + 6, ((unsigned)(props->MB_flag != 0) << 15) | ((unsigned)(props->ME_flag != 0) << 14), 2);
  be_put(h + 8, props->data_length, 8);
  memcpy(h + 16, props->type, strlen(props->type));
  if (fwrite(h, 1, HDR, w->fp) != HDR) return LIME_ERR_WRITE;
  w->first_record = 0;
  w->header_nextP = 0;
  w->isLastP = props->ME_flag;
  w->bytes_total = w->bytes_left = props->data_length;
  w->rec_ptr = 0;
  w->rec_start = (n_uint64_t)ftello(w->fp);
  w->bytes_pad = pad8(w->bytes_total);
  return LIME_SUCCESS;
}

int limeWriteRecordData(void *source, n_uint64_t *nbytes, LimeWriter *w)
{
  if (!source || !nbytes || !w || w->header_nextP) return LIME_ERR_PARAM;
  n_uint64_t n = *nbytes < w->bytes_left ? *nbytes : w->bytes_left;
  size_t put = fwrite(source, 1, (size_t)n, w->fp);
  w->rec_ptr += put;
  w->bytes_left -= put;
  *nbytes = put;
  if (put != n) return LIME_ERR_WRITE;
  if (w->bytes_left == 0) {  // the record is complete: pad it
    static const unsigned char zero[8];
    if (w->bytes_pad && fwrite(zero, 1, w->bytes_pad, w->fp) != w->bytes_pad) return LIME_ERR_WRITE;
    w->header_nextP = 1;
    if (w->isLastP) w->last_written = 1;
  }
  return LIME_SUCCESS;
}
