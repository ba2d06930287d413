// lime.cu -- LIME files: ILDG gauge configurations and ETMC spinor files,
// read and written the way qcd_lib does (lib/src/qcd_io.c:204-399 gauge
// read, :419-540 gauge write, :984-1150 spinor read, :1766-1950 spinor
// write), with the record layer written here from the LIME v1 format that
// c-lime implements (the c-lime headers qcd_lib vendors, include/lime_defs.h
// and include/lime_binary_header.h; c-lime itself is not in the tree).
//
// LIME record = 144-byte header + data + zero padding to a multiple of 8:
//   bytes 0-3   magic number 0x456789ab (big-endian)
//   bytes 4-5   version 1 (big-endian)
//   byte  6     flags: 0x80 message begin, 0x40 message end
//   bytes 8-15  data length in bytes (big-endian)
//   bytes 16-143 record type, NUL padded
// ILDG gauge data ("ildg-binary-data"): big-endian reals (precision 64 or 32
// from the "ildg-format" XML), order [t][z][y][x][mu'][row][col][re, im]
// with mu' = 0..3 the x, y, z, t links: qcd_lib's direction mu = (mu' + 1) % 4.
// ETMC spinor data ("scidac-binary-data" after an "etmc-propagator-format" or
// "etmc-source-format" XML record): big-endian, [t][z][y][x][spin][colour][re, im].
//
// The byte swapping and site reordering run on the GPU (one thread per link
// or site); the host only moves the file's bytes. qcd_lib's 32-bit gauge
// branch byte-swaps only the first time-slice's worth of floats
// (qcd_io.c:377); this reader swaps all of them.
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "internal.h"

namespace qg {

namespace {

struct LimeRec {
  std::string type;
  int64_t data_off;
  uint64_t len;
};

constexpr uint32_t kLimeMagic = 0x456789abu;
constexpr int kLimeHeader = 144;

uint64_t get_be(const unsigned char *p, int n)
{
  uint64_t v = 0;
  for (int i = 0; i < n; i++) v = (v << 8) | p[i];
  return v;
}
void put_be(unsigned char *p, uint64_t v, int n)
{
  for (int i = n - 1; i >= 0; i--) {
    p[i] = (unsigned char)(v & 0xffu);
    v >>= 8;
  }
}

bool lime_scan(FILE *f, std::vector<LimeRec> &recs)
{
  unsigned char h[kLimeHeader];
  int64_t pos = 0;
  if (fseeko(f, 0, SEEK_END) != 0) {
    set_error("LIME: cannot size the file");
    return false;
  }
  const int64_t fsize = (int64_t)ftello(f);
  while (true) {
    if (fseeko(f, pos, SEEK_SET) != 0) break;
    size_t n = fread(h, 1, kLimeHeader, f);
    if (n == 0) break;
    if (n != (size_t)kLimeHeader || get_be(h, 4) != kLimeMagic) {
      set_error("LIME: bad record header at byte %lld", (long long)pos);
      return false;
    }
    LimeRec r;
    r.len = get_be(h + 8, 8);
    r.type.assign((const char *)h + 16, strnlen((const char *)h + 16, 128));
    r.data_off = pos + kLimeHeader;
    // a corrupt length must not run past the file (nor overflow the next offset)
    if (r.len > (uint64_t)(fsize - r.data_off)) {
      set_error("LIME: record at byte %lld claims %llu bytes, past the end of the file", (long long)pos,
                (unsigned long long)r.len);
      return false;
    }
    recs.push_back(r);
    pos = r.data_off + (int64_t)((r.len + 7) / 8 * 8);
  }
  return true;
}

bool lime_put(FILE *f, const char *type, const void *data, uint64_t len, bool mb, bool me)
{
  unsigned char h[kLimeHeader];
  memset(h, 0, sizeof(h));
  put_be(h, kLimeMagic, 4);
  put_be(h + 4, 1, 2);
  h[6] = (unsigned char)((mb ? 0x80 : 0) | (me ? 0x40 : 0));
  put_be(h + 8, len, 8);
  strncpy((char *)h + 16, type, 128);
  static const unsigned char zeros[8] = {0};
  const size_t pad = (size_t)((len + 7) / 8 * 8 - len);
  return fwrite(h, 1, kLimeHeader, f) == (size_t)kLimeHeader && fwrite(data, 1, len, f) == len &&
         fwrite(zeros, 1, pad, f) == pad;
}

std::string read_record(FILE *f, const LimeRec &r)
{
  std::string s((size_t)r.len, '\0');
  if (fseeko(f, r.data_off, SEEK_SET) != 0 || fread(&s[0], 1, r.len, f) != r.len) return std::string();
  return s;
}

// the integer between <tag> and </tag> (white space allowed), or -1
long xml_int(const std::string &xml, const char *tag)
{
  const std::string open = std::string("<") + tag + ">";
  size_t p = xml.find(open);
  if (p == std::string::npos) return -1;
  return strtol(xml.c_str() + p + open.size(), nullptr, 10);
}

// the data of the first record of type `data_type` after a record of type
// `fmt_type`, its precision (32 or 64) from the format record's XML, and
// the lattice it declares (lx ly lz lt)
bool find_data(FILE *f, const char *fmt_type, const char *fmt_type2, const char *data_type, LimeRec *data, int *prec,
               long dims[4])
{
  std::vector<LimeRec> recs;
  if (!lime_scan(f, recs)) return false;
  bool have_fmt = false;
  for (const LimeRec &r : recs) {
    if (r.type == fmt_type || (fmt_type2 && r.type == fmt_type2)) {
      const std::string xml = read_record(f, r);
      *prec = (int)xml_int(xml, "precision");
      dims[0] = xml_int(xml, "lx");
      dims[1] = xml_int(xml, "ly");
      dims[2] = xml_int(xml, "lz");
      dims[3] = xml_int(xml, "lt");
      have_fmt = true;
    } else if (r.type == data_type && have_fmt) {
      *data = r;
      return true;
    }
  }
  set_error("LIME: no %s record after a %s record", data_type, fmt_type);
  return false;
}

__device__ __forceinline__ double be_real(const unsigned char *p, int prec)
{
  if (prec == 64) {
    const uint2 w = *(const uint2 *)p;  // bytes b0..b7 of a big-endian double
    const unsigned hi = __byte_perm(w.x, 0, 0x0123), lo = __byte_perm(w.y, 0, 0x0123);
    return __hiloint2double((int)hi, (int)lo);
  }
  const unsigned w = __byte_perm(*(const unsigned *)p, 0, 0x0123);
  return (double)__uint_as_float(w);
}

__device__ __forceinline__ void be_store(unsigned char *p, double v)
{
  const unsigned hi = (unsigned)__double2hiint(v), lo = (unsigned)__double2loint(v);
  *(uint2 *)p = make_uint2(__byte_perm(hi, 0, 0x0123), __byte_perm(lo, 0, 0x0123));
}

struct Dims {
  int L[4];  // t, x, y, z
};

// file link i = ((((t * Lz + z) * Ly + y) * Lx + x) * 4 + mu') -> host layout
__global__ void k_ildg_to_aos(double *dst, const unsigned char *src, Dims d, int64_t nlinks, int prec)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlinks) return;
  const int mf = (int)(i & 3);
  int64_t s = i >> 2;
  const int x = (int)(s % d.L[1]);
  s /= d.L[1];
  const int y = (int)(s % d.L[2]);
  s /= d.L[2];
  const int z = (int)(s % d.L[3]);
  const int t = (int)(s / d.L[3]);
  const int64_t site = t + (int64_t)d.L[0] * (x + (int64_t)d.L[1] * (y + (int64_t)d.L[2] * z));
  const int nu = (mf + 1) & 3;
  const int w = prec / 8;
#pragma unroll
  for (int k = 0; k < 18; k++) dst[(site * 4 + nu) * 18 + k] = be_real(src + (i * 18 + k) * w, prec);
}

__global__ void k_aos_to_ildg(unsigned char *dst, const double *src, Dims d, int64_t nlinks)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nlinks) return;
  const int mf = (int)(i & 3);
  int64_t s = i >> 2;
  const int x = (int)(s % d.L[1]);
  s /= d.L[1];
  const int y = (int)(s % d.L[2]);
  s /= d.L[2];
  const int z = (int)(s % d.L[3]);
  const int t = (int)(s / d.L[3]);
  const int64_t site = t + (int64_t)d.L[0] * (x + (int64_t)d.L[1] * (y + (int64_t)d.L[2] * z));
  const int nu = (mf + 1) & 3;
#pragma unroll
  for (int k = 0; k < 18; k++) be_store(dst + (i * 18 + k) * 8, src[(site * 4 + nu) * 18 + k]);
}

// file site i = ((t * Lz + z) * Ly + y) * Lx + x -> host layout (24 reals)
__global__ void k_etmc_to_aos(double *dst, const unsigned char *src, Dims d, int64_t nsites, int prec)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsites) return;
  int64_t s = i;
  const int x = (int)(s % d.L[1]);
  s /= d.L[1];
  const int y = (int)(s % d.L[2]);
  s /= d.L[2];
  const int z = (int)(s % d.L[3]);
  const int t = (int)(s / d.L[3]);
  const int64_t site = t + (int64_t)d.L[0] * (x + (int64_t)d.L[1] * (y + (int64_t)d.L[2] * z));
  const int w = prec / 8;
#pragma unroll
  for (int k = 0; k < 24; k++) dst[site * 24 + k] = be_real(src + (i * 24 + k) * w, prec);
}

__global__ void k_aos_to_etmc(unsigned char *dst, const double *src, Dims d, int64_t nsites)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsites) return;
  int64_t s = i;
  const int x = (int)(s % d.L[1]);
  s /= d.L[1];
  const int y = (int)(s % d.L[2]);
  s /= d.L[2];
  const int z = (int)(s % d.L[3]);
  const int t = (int)(s / d.L[3]);
  const int64_t site = t + (int64_t)d.L[0] * (x + (int64_t)d.L[1] * (y + (int64_t)d.L[2] * z));
#pragma unroll
  for (int k = 0; k < 24; k++) be_store(dst + (i * 24 + k) * 8, src[site * 24 + k]);
}

// pinned host + device byte buffers of one file's data
struct Bytes {
  void *host = nullptr, *dev = nullptr;
  ~Bytes()
  {
    if (host) cudaFreeHost(host);
    if (dev) cudaFree(dev);
  }
  bool alloc(size_t n) { return QG_CUDA(cudaMallocHost(&host, n)) && QG_CUDA(cudaMalloc(&dev, n)); }
};

struct File {
  FILE *f;
  explicit File(const char *name, const char *mode) : f(fopen(name, mode)) {}
  ~File()
  {
    if (f) fclose(f);
  }
};

bool read_payload(const char *fname, const int L[4], const char *fmt, const char *fmt2, const char *data_type,
                  uint64_t reals, Bytes &b, int *prec)
{
  File file(fname, "rb");
  if (!file.f) {
    set_error("LIME: cannot open %s for reading", fname);
    return false;
  }
  LimeRec r;
  long dims[4];
  if (!find_data(file.f, fmt, fmt2, data_type, &r, prec, dims)) return false;
  if (*prec != 32 && *prec != 64) {
    set_error("LIME: unsupported precision %d in %s", *prec, fname);
    return false;
  }
  if ((dims[0] >= 0 && dims[0] != L[1]) || (dims[1] >= 0 && dims[1] != L[2]) || (dims[2] >= 0 && dims[2] != L[3]) ||
      (dims[3] >= 0 && dims[3] != L[0])) {
    set_error("LIME: %s holds a %ldx%ldx%ldx%ld lattice (x y z t)", fname, dims[0], dims[1], dims[2], dims[3]);
    return false;
  }
  const uint64_t need = reals * (uint64_t)(*prec / 8);
  if (r.len < need) {
    set_error("LIME: %s: %llu data bytes, %llu expected", fname, (unsigned long long)r.len,
              (unsigned long long)need);
    return false;
  }
  if (!b.alloc(need)) return false;
  if (fseeko(file.f, r.data_off, SEEK_SET) != 0 || fread(b.host, 1, need, file.f) != need) {
    set_error("LIME: short read of %s", fname);
    return false;
  }
  return QG_CUDA(cudaMemcpyAsync(b.dev, b.host, need, cudaMemcpyHostToDevice, stream()));
}

}  // namespace

bool lime_read_gauge(const char *fname, const int L[4], void *dev_aos)
{
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  Bytes b;
  int prec = 0;
  if (!read_payload(fname, L, "ildg-format", nullptr, "ildg-binary-data", (uint64_t)V * 72, b, &prec)) return false;
  Dims d;
  memcpy(d.L, L, sizeof(d.L));
  const int64_t n = V * 4;
  k_ildg_to_aos<<<(unsigned)((n + 127) / 128), 128, 0, stream()>>>((double *)dev_aos, (const unsigned char *)b.dev,
                                                                    d, n, prec);
  return QG_LAUNCHED("ildg_to_aos") && QG_CUDA(cudaStreamSynchronize(stream()));
}

bool lime_write_gauge(const char *fname, const int L[4], const void *dev_aos, const char *message)
{
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  const uint64_t bytes = (uint64_t)V * 72 * 8;
  Bytes b;
  if (!b.alloc(bytes)) return false;
  Dims d;
  memcpy(d.L, L, sizeof(d.L));
  const int64_t n = V * 4;
  k_aos_to_ildg<<<(unsigned)((n + 127) / 128), 128, 0, stream()>>>((unsigned char *)b.dev, (const double *)dev_aos,
                                                                    d, n);
  if (!QG_LAUNCHED("aos_to_ildg") ||
      !QG_CUDA(cudaMemcpyAsync(b.host, b.dev, bytes, cudaMemcpyDeviceToHost, stream())) ||
      !QG_CUDA(cudaStreamSynchronize(stream())))
    return false;
  char xml[1024];
  snprintf(xml, sizeof(xml),
           "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n<ildgFormat xmlns=\"http://www.lqcd.org/ildg\"\n"
           "            xmlns:xsi=\"http://www.w3.org/2001/XMLSchema-instance\"\n"
           "            xsi:schemaLocation=\"http://www.lqcd.org/ildg filefmt.xsd\">\n  <version> 1.0 </version>\n"
           "  <field> su3gauge </field>\n  <precision> 64 </precision>\n  <lx> %d </lx>\n  <ly> %d </ly>\n"
           "  <lz> %d </lz>\n  <lt> %d </lt>\n</ildgFormat>",
           L[1], L[2], L[3], L[0]);
  File file(fname, "wb");
  const char *msg = message ? message : "";
  if (!file.f || !lime_put(file.f, "ildg-format", xml, strlen(xml), true, false) ||
      !lime_put(file.f, "xlf-info", msg, strlen(msg), false, false) ||
      !lime_put(file.f, "ildg-binary-data", b.host, bytes, false, true)) {
    set_error("LIME: cannot write %s", fname);
    return false;
  }
  return true;
}

bool lime_read_spinor(const char *fname, const int L[4], void *dev_aos)
{
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  Bytes b;
  int prec = 0;
  if (!read_payload(fname, L, "etmc-propagator-format", "etmc-source-format", "scidac-binary-data", (uint64_t)V * 24,
                    b, &prec))
    return false;
  Dims d;
  memcpy(d.L, L, sizeof(d.L));
  k_etmc_to_aos<<<(unsigned)((V + 127) / 128), 128, 0, stream()>>>((double *)dev_aos, (const unsigned char *)b.dev,
                                                                    d, V, prec);
  return QG_LAUNCHED("etmc_to_aos") && QG_CUDA(cudaStreamSynchronize(stream()));
}

bool lime_write_spinor(const char *fname, const int L[4], const void *dev_aos, bool source)
{
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  const uint64_t bytes = (uint64_t)V * 24 * 8;
  Bytes b;
  if (!b.alloc(bytes)) return false;
  Dims d;
  memcpy(d.L, L, sizeof(d.L));
  k_aos_to_etmc<<<(unsigned)((V + 127) / 128), 128, 0, stream()>>>((unsigned char *)b.dev, (const double *)dev_aos,
                                                                    d, V);
  if (!QG_LAUNCHED("aos_to_etmc") ||
      !QG_CUDA(cudaMemcpyAsync(b.host, b.dev, bytes, cudaMemcpyDeviceToHost, stream())) ||
      !QG_CUDA(cudaStreamSynchronize(stream())))
    return false;
  const char *kind = source ? "DiracFermion_Source" : "DiracFermion_Sink";
  char xml[1024];
  snprintf(xml, sizeof(xml),
           "<?xml version=\"1.0\" encoding=\"UTF-8\"?>\n<etmcFormat>\n\t<field>diracFermion</field>\n"
           "\t<precision>64</precision>\n\t<flavours>1</flavours>\n\t<lx>%d</lx>\n\t<ly>%d</ly>\n\t<lz>%d</lz>\n"
           "\t<lt>%d</lt>\n\t<spin>4</spin>\n\t<colour>3</colour>\n</etmcFormat>",
           L[1], L[2], L[3], L[0]);
  File file(fname, "wb");
  if (!file.f || !lime_put(file.f, source ? "source-type" : "propagator-type", kind, strlen(kind), true, true) ||
      !lime_put(file.f, source ? "etmc-source-format" : "etmc-propagator-format", xml, strlen(xml), true, true) ||
      !lime_put(file.f, "scidac-binary-data", b.host, bytes, true, true)) {
    set_error("LIME: cannot write %s", fname);
    return false;
  }
  return true;
}

// Legacy propagator vector files (lib/src/qcd_io.c:907-1340, dispatcher
// :1386). All three hold big-endian reals in the order [x][y][z][t][spin]
// [colour][re, im] (x slowest, t fastest): CMI (type 0) float32 with no
// header; HMC (type 1) an ASCII line "beta kappa mu L T" and then float64
// data of all twelve source columns, column nu * 3 + c2 at (nu * 3 + c2) x 24 V
// reals after the line; HMCV (type 2) the same line and one column.
// file site i = ((x * Ly + y) * Lz + z) * Lt + t -> host layout (24 reals)
__global__ void k_xyzt_to_aos(double *dst, const unsigned char *src, Dims d, int64_t nsites, int prec)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsites) return;
  int64_t s = i;
  const int t = (int)(s % d.L[0]);
  s /= d.L[0];
  const int z = (int)(s % d.L[3]);
  s /= d.L[3];
  const int y = (int)(s % d.L[2]);
  const int x = (int)(s / d.L[2]);
  const int64_t site = t + (int64_t)d.L[0] * (x + (int64_t)d.L[1] * (y + (int64_t)d.L[2] * z));
  const int w = prec / 8;
#pragma unroll
  for (int k = 0; k < 24; k++) dst[site * 24 + k] = be_real(src + (i * 24 + k) * w, prec);
}

// host layout -> CMI file order, big-endian float32 (rounded to nearest
// as qcd_writeVectorCMI's double-to-float assignment, qcd_io.c:1741-1750)
__global__ void k_aos_to_xyzt32(unsigned char *dst, const double *src, Dims d, int64_t nsites)
{
  const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nsites) return;
  int64_t s = i;
  const int t = (int)(s % d.L[0]);
  s /= d.L[0];
  const int z = (int)(s % d.L[3]);
  s /= d.L[3];
  const int y = (int)(s % d.L[2]);
  const int x = (int)(s / d.L[2]);
  const int64_t site = t + (int64_t)d.L[0] * (x + (int64_t)d.L[1] * (y + (int64_t)d.L[2] * z));
#pragma unroll
  for (int k = 0; k < 24; k++)
    *(unsigned *)(dst + (i * 24 + k) * 4) = __byte_perm(__float_as_uint((float)src[site * 24 + k]), 0, 0x0123);
}

bool cmi_write_spinor(const char *fname, const int L[4], const void *dev_aos)
{
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  const uint64_t bytes = (uint64_t)V * 24 * 4;
  Bytes b;
  if (!b.alloc(bytes)) return false;
  Dims d;
  memcpy(d.L, L, sizeof(d.L));
  k_aos_to_xyzt32<<<(unsigned)((V + 127) / 128), 128, 0, stream()>>>((unsigned char *)b.dev, (const double *)dev_aos,
                                                                      d, V);
  if (!QG_LAUNCHED("aos_to_xyzt32") ||
      !QG_CUDA(cudaMemcpyAsync(b.host, b.dev, bytes, cudaMemcpyDeviceToHost, stream())) ||
      !QG_CUDA(cudaStreamSynchronize(stream())))
    return false;
  File file(fname, "wb");
  if (!file.f) {
    set_error("process 0: Error in qcd_writeVectorCMI! Cannot open %s for writing", fname);
    return false;
  }
  if (fwrite(b.host, 1, bytes, file.f) != bytes) {
    set_error("qcd_writeVectorCMI: short write to %s", fname);
    return false;
  }
  return true;
}

bool legacy_read_spinor(const char *fname, const int L[4], int type, int col, void *dev_aos)
{
  const char *name = type == 0 ? "qcd_getVectorCMI" : type == 1 ? "qcd_getVectorHMC" : "qcd_getVectorHMCV";
  if (type < 0 || type > 2 || col < 0 || col > 11) {
    set_error("%s: type 0..2 and a source column 0..11", name);
    return false;
  }
  File file(fname, "rb");
  if (!file.f) {
    set_error("%s! Cannot open %s for reading", name, fname);
    return false;
  }
  const int64_t V = (int64_t)L[0] * L[1] * L[2] * L[3];
  const int prec = type == 0 ? 32 : 64;
  int64_t off = 0;
  if (type != 0) {  // the header line, read as the reference reads it
    double beta, kappa, mu;
    int fL = -1, fT = -1;
    if (fscanf(file.f, "%lf %lf %lf %d %d\n", &beta, &kappa, &mu, &fL, &fT) != 5 || fL != L[1] || fT != L[0]) {
      set_error("%s! Dimensions in file %s don't match geometry!", name, fname);
      return false;
    }
    off = (int64_t)ftello(file.f);
    if (type == 1) off += (int64_t)col * 24 * V * 8;
  }
  const uint64_t need = (uint64_t)V * 24 * (prec / 8);
  if (fseeko(file.f, 0, SEEK_END) != 0 || (int64_t)ftello(file.f) < off + (int64_t)need) {
    set_error("%s! %s is shorter than a %lldx%lldx%lldx%lld vector%s", name, fname, (long long)L[1],
              (long long)L[2], (long long)L[3], (long long)L[0], type == 1 ? " column" : "");
    return false;
  }
  Bytes b;
  if (!b.alloc(need)) return false;
  if (fseeko(file.f, off, SEEK_SET) != 0 || fread(b.host, 1, need, file.f) != need) {
    set_error("%s! short read of %s", name, fname);
    return false;
  }
  if (!QG_CUDA(cudaMemcpyAsync(b.dev, b.host, need, cudaMemcpyHostToDevice, stream()))) return false;
  Dims d;
  memcpy(d.L, L, sizeof(d.L));
  k_xyzt_to_aos<<<(unsigned)((V + 127) / 128), 128, 0, stream()>>>((double *)dev_aos, (const unsigned char *)b.dev,
                                                                    d, V, prec);
  return QG_LAUNCHED("legacy_to_aos") && QG_CUDA(cudaStreamSynchronize(stream()));
}

}  // namespace qg

namespace qg {
namespace {
struct DevBuf {
  void *p = nullptr;
  ~DevBuf()
  {
    if (p) {
      cudaStreamSynchronize(stream());
      cudaFree(p);
    }
  }
  bool alloc(size_t n) { return QG_CUDA(cudaMalloc(&p, n)); }
};
}  // namespace
}  // namespace qg

extern "C" {

int qcdgpu_gauge_load_lime(qcdgpu_gauge g, const char *fname)
{
  qg::DevBuf b;
  if (!g || !fname || !b.alloc((size_t)g->V * 72 * sizeof(double)) || !qg::lime_read_gauge(fname, g->L, b.p))
    return 1;
  qg::gauge_forget(g);
  return qg::pack_gauge(g, b.p) ? 0 : 1;
}

int qcdgpu_gauge_save_lime(qcdgpu_gauge g, const char *fname, const char *message)
{
  qg::DevBuf b;
  if (!g || !fname || !b.alloc((size_t)g->V * 72 * sizeof(double)) || !qg::gauge_to_aos_dev(g, b.p)) return 1;
  return qg::lime_write_gauge(fname, g->L, b.p, message) ? 0 : 1;
}

int qcdgpu_field_load_lime(qcdgpu_field f, const char *fname)
{
  qg::DevBuf b;
  if (!f || !fname || !b.alloc((size_t)f->V * 24 * sizeof(double)) || !qg::lime_read_spinor(fname, f->L, b.p))
    return 1;
  return qg::spinor_from_aos_dev(f, b.p) && QG_CUDA(cudaStreamSynchronize(qg::stream())) ? 0 : 1;
}

int qcdgpu_field_save_lime(qcdgpu_field f, const char *fname, int source)
{
  qg::DevBuf b;
  if (!f || !fname || !b.alloc((size_t)f->V * 24 * sizeof(double)) || !qg::spinor_to_aos_dev(f, b.p)) return 1;
  return qg::lime_write_spinor(fname, f->L, b.p, source != 0) ? 0 : 1;
}

}  // extern "C"
