// Driver for the reference's own file readers (TEST INFRASTRUCTURE, built by
// oracle/build_ref.sh into oracle/_ref/libscreaders.so): the readers of
// Source/sc_readdata.cpp compiled as they are, with the Qt stand-ins of
// oracle/ref_stubs_io and the console widImage stand-in of
// ref_stubs_io/readers_env.h forced in ahead of them. A read image keeps its
// extents, data (x inner, y outer) and meta information in reading order.
#include <cstdlib>
#include <new>

#include "sc_readdata.h"

// The reference's EDF loops run one record past the data they read
// (nn <= RecRead/size) and so write the image element genIDX(rows*cols) = -1,
// just before its `new double[]` array. Array allocations of this library
// carry 64 bytes of slack in front, which that write lands in instead of the
// allocator's bookkeeping; the reader's results are unchanged.
void *operator new[](std::size_t n) {
    char *p = (char *)std::malloc(n + 64);
    if (!p) throw std::bad_alloc();
    return p + 64;
}
void operator delete[](void *p) noexcept {
    if (p) std::free((char *)p - 64);
}
void operator delete[](void *p, std::size_t) noexcept {
    if (p) std::free((char *)p - 64);
}

static widImage *cs_add(int x0, int x1, int y0, int y1, double *d, QString title) {
    widImage *w = new widImage;
    w->setData(x0, x1, y0, y1, d);
    w->title = title;
    return w;
}

extern "C" {

// kind: "kws", "edf", "spreadsheet", "sascrystal", "tiff", "2dsans" (its text
// forms: the XML stand-in reads nothing); null when the reader
// returns none
void *ref_read_image(const char *kind, const char *fn) {
    const QString k(kind), f(fn);
    if (k == "kws") return SC_ReadData::readImageKWSData(cs_add, f);
    if (k == "edf") return SC_ReadData::readImageEDF(cs_add, f);
    if (k == "spreadsheet") return SC_ReadData::readImageSpreadsheet(cs_add, f);
    if (k == "sascrystal") return SC_ReadData::readImageSasCrystal(cs_add, f);
    if (k == "tiff") return SC_ReadData::readImageTiff(cs_add, f);
    if (k == "2dsans") return SC_ReadData::readImage2dSans(cs_add, f);
    return nullptr;
}

void ref_image_dims(void *h, int *d) {
    widImage *w = (widImage *)h;
    d[0] = w->minX;
    d[1] = w->maxX;
    d[2] = w->minY;
    d[3] = w->maxY;
}

long ref_image_data(void *h, double *out, long cap) {
    widImage *w = (widImage *)h;
    const long n = (long)w->data.size();
    for (long i = 0; i < n && i < cap; i++) out[i] = w->data[(size_t)i];
    return n;
}

int ref_image_meta_count(void *h) { return (int)((widImage *)h)->metaKeys.size(); }
const char *ref_image_meta_key(void *h, int i) { return ((widImage *)h)->metaKeys[(size_t)i].c_str(); }
const char *ref_image_meta_value(void *h, int i) { return ((widImage *)h)->metaVals[(size_t)i].c_str(); }
const char *ref_image_title(void *h) { return ((widImage *)h)->title.c_str(); }

// an image from raw data (x inner, y outer), for findBeamCenter
void *ref_image_from_data(int x0, int x1, int y0, int y1, const double *d) {
    return cs_add(x0, x1, y0, y1, const_cast<double *>(d), QString("data"));
}

// findBeamCenter from the start point (x0, y0) (the image's centre entries)
void ref_find_beam_center(void *h, int x0, int y0, int *xerg, int *yerg) {
    widImage *w = (widImage *)h;
    w->fileInfos.centerX = x0;
    w->fileInfos.centerY = y0;
    SC_ReadData::findBeamCenter(w, *xerg, *yerg);
}

void ref_image_free(void *h) { delete (widImage *)h; }
}
