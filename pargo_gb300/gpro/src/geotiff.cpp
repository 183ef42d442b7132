// geotiff.cpp -- the GeoTIFF reading and writing RasterLayer needs, without GDAL.
//
// Reads classic TIFF (32-bit offsets) and BigTIFF (64-bit offsets), either
// byte order, one sample per pixel, uncompressed strips or tiles of
// 8/16/32/64-bit integer or IEEE float samples; the georeferencing is taken
// from ModelPixelScale (33550) and ModelTiepoint (33922) as a GDAL
// geotransform, nodata from GDAL_NODATA (42113); the GeoKey tags
// (34735-34737) are carried through untouched.  Writes little-endian
// uncompressed float32 or float64 strips with the same tags, as the
// reference's GTiff output (gpro/rasterLayer.h:957-995) carries them: classic
// TIFF below 4 GB, BigTIFF above (a 32768^2 float32 raster is 4 GB), as GDAL
// chooses for uncompressed output.
// The file is read in one call and decoded a strip or tile row at a time (rows
// of a little-endian file as plain copies on a little-endian host); the writer
// streams its samples through a fixed buffer after the header.
#include <cstdio>

#include "gpro/gpro.h"

namespace GPRO {

namespace {

struct Reader {
    const std::vector<unsigned char>& b;
    bool big;
    uint16_t u16(size_t o) const {
        return big ? (uint16_t)(b[o] << 8 | b[o + 1]) : (uint16_t)(b[o] | b[o + 1] << 8);
    }
    uint32_t u32(size_t o) const {
        return big ? ((uint32_t)b[o] << 24 | (uint32_t)b[o + 1] << 16 | (uint32_t)b[o + 2] << 8 | b[o + 3])
                   : ((uint32_t)b[o] | (uint32_t)b[o + 1] << 8 | (uint32_t)b[o + 2] << 16 | (uint32_t)b[o + 3] << 24);
    }
    uint64_t u64(size_t o) const {
        return big ? ((uint64_t)u32(o) << 32 | u32(o + 4)) : ((uint64_t)u32(o + 4) << 32 | u32(o));
    }
};

struct Entry {
    uint16_t tag = 0, type = 0;
    uint32_t count = 0;
    size_t off = 0;  // where the values are (inline or out of line)
};

size_t type_size(uint16_t t) {
    switch (t) {
        case 1: case 2: case 6: case 7: return 1;
        case 3: case 8: return 2;
        case 4: case 9: case 11: case 13: return 4;
        case 5: case 10: case 12: case 16: case 17: case 18: return 8;  // 16-18: BigTIFF's 64-bit integers
        default: return 0;
    }
}

double sample(const Reader& r, size_t o, int bits, int fmt) {
    switch (bits) {
        case 8: return fmt == 2 ? (double)(int8_t)r.b[o] : (double)r.b[o];
        case 16: return fmt == 2 ? (double)(int16_t)r.u16(o) : (double)r.u16(o);
        case 32: {
            const uint32_t v = r.u32(o);
            if (fmt == 3) {
                float f;
                memcpy(&f, &v, 4);
                return f;
            }
            return fmt == 2 ? (double)(int32_t)v : (double)v;
        }
        default: {
            const uint64_t v = r.u64(o);
            if (fmt == 3) {
                double d;
                memcpy(&d, &v, 8);
                return d;
            }
            return fmt == 2 ? (double)(int64_t)v : (double)v;
        }
    }
}

// Little-endian host: samples of a little-endian file are copied as they lie.
bool host_little_endian() {
    const uint16_t one = 1;
    unsigned char c;
    memcpy(&c, &one, 1);
    return c == 1;
}

// n consecutive samples starting at byte o into dst; the same values as
// sample() one by one, with the common little-endian cases as plain copies.
void samples(const Reader& r, size_t o, size_t n, int bits, int fmt, double* dst) {
    const unsigned char* p = r.b.data() + o;
    if (!r.big && host_little_endian()) {
        if (bits == 32 && fmt == 3) {
            for (size_t k = 0; k < n; k++) {
                float v;
                memcpy(&v, p + 4 * k, 4);
                dst[k] = v;
            }
            return;
        }
        if (bits == 64 && fmt == 3) {
            memcpy(dst, p, 8 * n);
            return;
        }
        if (bits == 16 && fmt == 2) {
            for (size_t k = 0; k < n; k++) {
                int16_t v;
                memcpy(&v, p + 2 * k, 2);
                dst[k] = v;
            }
            return;
        }
        if (bits == 32 && fmt == 2) {
            for (size_t k = 0; k < n; k++) {
                int32_t v;
                memcpy(&v, p + 4 * k, 4);
                dst[k] = v;
            }
            return;
        }
    }
    for (size_t k = 0; k < n; k++) dst[k] = sample(r, o + k * ((size_t)bits / 8), bits, fmt);
}

}  // namespace

bool read_geotiff(const char* path, GeoRaster* out, std::string* err) {
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    if (!f) {
        *err = std::string("cannot open ") + path;
        return false;
    }
    const std::streamoff fsize = f.tellg();
    std::vector<unsigned char> b(fsize > 0 ? (size_t)fsize : 0);
    f.seekg(0);
    if (!b.empty() && !f.read(reinterpret_cast<char*>(b.data()), (std::streamsize)b.size())) {
        *err = std::string(path) + ": read failed";
        return false;
    }
    if (b.size() < 8 || !((b[0] == 'I' && b[1] == 'I') || (b[0] == 'M' && b[1] == 'M'))) {
        *err = std::string(path) + ": not a TIFF file";
        return false;
    }
    Reader r{b, b[0] == 'M'};
    // classic TIFF (42: 32-bit offsets, 12-byte entries) or BigTIFF (43:
    // 64-bit offsets and counts, 20-byte entries, values of up to 8 bytes inline)
    const uint16_t version = r.u16(2);
    const bool bigtiff = version == 43;
    if (version != 42 && !(bigtiff && b.size() >= 16 && r.u16(4) == 8 && r.u16(6) == 0)) {
        *err = std::string(path) + ": only classic TIFF and BigTIFF are supported";
        return false;
    }
    const uint64_t ifd = bigtiff ? r.u64(8) : r.u32(4);
    const size_t count_bytes = bigtiff ? 8 : 2, entry_bytes = bigtiff ? 20 : 12, inline_bytes = bigtiff ? 8 : 4;
    if (ifd > b.size() || ifd + count_bytes > b.size()) {
        *err = std::string(path) + ": truncated";
        return false;
    }
    const uint64_t n = bigtiff ? r.u64(ifd) : r.u16(ifd);
    std::vector<Entry> es;
    for (uint64_t i = 0; i < n && i < 65536; i++) {
        const size_t e = ifd + count_bytes + entry_bytes * i;
        if (e + entry_bytes > b.size()) break;
        Entry x;
        x.tag = r.u16(e);
        x.type = r.u16(e + 2);
        const uint64_t count = bigtiff ? r.u64(e + 4) : r.u32(e + 4);
        if (count > b.size()) continue;  // more values than the file has bytes
        x.count = (uint32_t)count;
        const size_t bytes = type_size(x.type) * (size_t)count;
        const size_t vo = e + (bigtiff ? 12 : 8);
        x.off = bytes <= inline_bytes ? vo : (size_t)(bigtiff ? r.u64(vo) : r.u32(vo));
        if (x.off > b.size() || bytes > b.size() - x.off) continue;
        es.push_back(x);
    }
    auto find = [&](uint16_t tag) -> const Entry* {
        for (auto& e : es)
            if (e.tag == tag) return &e;
        return nullptr;
    };
    auto num = [&](const Entry* e, uint32_t k) -> double {
        if (k >= e->count) return 0.0;  // past the tag's values
        switch (e->type) {
            case 3: return r.u16(e->off + 2 * k);
            case 4: return r.u32(e->off + 4 * k);
            case 16: return (double)r.u64(e->off + 8 * k);
            case 12: {
                uint64_t v = r.u64(e->off + 8 * k);
                double d;
                memcpy(&d, &v, 8);
                return d;
            }
            case 1: return b[e->off + k];
            default: return 0.0;
        }
    };
    const Entry* w = find(256);
    const Entry* h = find(257);
    if (!w || !h) {
        *err = std::string(path) + ": missing image size";
        return false;
    }
    GeoRaster g;
    const double wd = num(w, 0), hd = num(h, 0);
    if (!(wd >= 1 && hd >= 1 && wd <= 2147483647.0 && hd <= 2147483647.0 && wd * hd <= 68719476736.0)) {
        *err = std::string(path) + ": bad image size";
        return false;
    }
    g.cols = (int)wd;
    g.rows = (int)hd;
    const Entry* bps = find(258);
    const int bits = bps ? (int)num(bps, 0) : 1;
    const Entry* sf = find(339);
    const int fmt = sf ? (int)num(sf, 0) : 1;
    const Entry* comp = find(259);
    const Entry* spp = find(277);
    if ((comp && num(comp, 0) != 1) || (spp && num(spp, 0) != 1) ||
        !(bits == 8 || bits == 16 || bits == 32 || bits == 64) || (fmt == 3 && bits < 32)) {
        *err = std::string(path) + ": only uncompressed single-band 8/16/32/64-bit rasters are supported";
        return false;
    }
    g.dtype = fmt == 3 ? (bits == 32 ? PARGO_F32 : PARGO_F64) : (bits == 8 ? PARGO_I8 : bits == 16 ? PARGO_I16 : PARGO_I32);
    const size_t bpp = (size_t)bits / 8;
    g.values.assign((size_t)g.rows * g.cols, 0.0);
    const Entry* so = find(273);
    const Entry* to = find(324);
    if (so) {
        const Entry* rps = find(278);
        const Entry* sbc = find(279);
        const double per_d = rps ? num(rps, 0) : 0.0;
        const int64_t per = per_d >= 1 && per_d < g.rows ? (int64_t)per_d : g.rows;  // absent or too large: one strip
        for (uint32_t s = 0; s < so->count; s++) {
            const size_t base = (size_t)num(so, s);
            const int64_t r0 = (int64_t)s * per;
            const int64_t nr = std::min<int64_t>(per, g.rows - r0);
            if (nr <= 0) break;  // strips past the last row carry nothing
            const size_t need = (size_t)nr * g.cols * bpp;
            if (sbc && (size_t)num(sbc, s) < need) {
                *err = std::string(path) + ": short strip";
                return false;
            }
            if (base > b.size() || need > b.size() - base) {
                *err = std::string(path) + ": truncated strip";
                return false;
            }
            samples(r, base, (size_t)nr * g.cols, bits, fmt, g.values.data() + (size_t)r0 * g.cols);
        }
    } else if (to) {
        const Entry* tw = find(322);
        const Entry* tl = find(323);
        if (!tw || !tl) {
            *err = std::string(path) + ": tile size missing";
            return false;
        }
        const double twd = num(tw, 0), tld = num(tl, 0);
        if (!(twd >= 1 && tld >= 1 && twd <= 65536.0 && tld <= 65536.0)) {
            *err = std::string(path) + ": bad tile size";
            return false;
        }
        const int TW = (int)twd, TL = (int)tld;
        const int across = (g.cols + TW - 1) / TW;
        for (uint32_t t = 0; t < to->count; t++) {
            const size_t base = (size_t)num(to, t);
            const int64_t ty = (int64_t)t / across, tx = (int64_t)t % across;
            if (base > b.size() || (size_t)TW * TL * bpp > b.size() - base) {
                *err = std::string(path) + ": truncated tile";
                return false;
            }
            const int64_t nc = std::min<int64_t>(TW, g.cols - tx * TW);
            for (int64_t i = 0; i < TL && ty * TL + i < g.rows; i++)
                samples(r, base + (size_t)i * TW * bpp, (size_t)nc, bits, fmt,
                        g.values.data() + (size_t)(ty * TL + i) * g.cols + (size_t)tx * TW);
        }
    } else {
        *err = std::string(path) + ": no strips or tiles";
        return false;
    }
    const Entry* scale = find(33550);
    const Entry* tie = find(33922);
    if (scale && scale->count >= 2 && tie && tie->count >= 6) {
        const double sx = num(scale, 0), sy = num(scale, 1);
        const double ti = num(tie, 0), tj = num(tie, 1), tx = num(tie, 3), ty = num(tie, 4);
        const double t[6] = {tx - ti * sx, sx, 0.0, ty + tj * sy, 0.0, -sy};
        memcpy(g.transform, t, sizeof(t));
    }
    // the GeoKey tags and GDAL_NODATA, when they have their usual types
    // (SHORT, DOUBLE, ASCII; entries were kept only with their values inside the file)
    const Entry* gk = find(34735);
    if (gk && gk->type == 3) g.geokeys.assign(b.begin() + gk->off, b.begin() + gk->off + 2 * (size_t)gk->count);
    const Entry* gd = find(34736);
    if (gd && gd->type == 12) g.geodoubles.assign(b.begin() + gd->off, b.begin() + gd->off + 8 * (size_t)gd->count);
    const Entry* ga = find(34737);
    if (ga && ga->type == 2) g.geoascii.assign((const char*)b.data() + ga->off, ga->count);
    const Entry* gn = find(42113);
    if (gn && gn->type == 2) {
        std::string s((const char*)b.data() + gn->off, gn->count);
        g.nodata = atof(s.c_str());
        g.has_nodata = true;
    }
    if (r.big) {  // carried tags are written little-endian
        for (size_t k = 0; k + 1 < g.geokeys.size(); k += 2) std::swap(g.geokeys[k], g.geokeys[k + 1]);
        for (size_t k = 0; k + 7 < g.geodoubles.size(); k += 8) std::reverse(g.geodoubles.begin() + k, g.geodoubles.begin() + k + 8);
    }
    *out = std::move(g);
    return true;
}

namespace {

struct Writer {
    struct E {
        uint16_t tag, type;
        uint64_t count;
        std::vector<unsigned char> data;
    };
    std::vector<E> entries;
    void add(uint16_t tag, uint16_t type, uint64_t count, const void* data, size_t bytes) {
        E e{tag, type, count, std::vector<unsigned char>((const unsigned char*)data, (const unsigned char*)data + bytes)};
        entries.push_back(e);
    }
    void u16(uint16_t tag, uint16_t v) { add(tag, 3, 1, &v, 2); }
    void u32(uint16_t tag, uint32_t v) { add(tag, 4, 1, &v, 4); }
};

void put16(std::vector<unsigned char>& o, uint16_t v) {
    o.push_back(v & 0xff);
    o.push_back(v >> 8);
}
void put32(std::vector<unsigned char>& o, uint32_t v) {
    for (int k = 0; k < 4; k++) o.push_back((v >> (8 * k)) & 0xff);
}
void put64(std::vector<unsigned char>& o, uint64_t v) {
    for (int k = 0; k < 8; k++) o.push_back((v >> (8 * k)) & 0xff);
}

}  // namespace

bool write_geotiff(const char* path, const GeoRaster& m, const double* values, int dtype, std::string* err,
                   bool force_bigtiff) {
    const size_t bpp = dtype == PARGO_F32 ? 4 : 8;
    const size_t rowbytes = (size_t)m.cols * bpp;
    const uint64_t total = (uint64_t)rowbytes * m.rows;
    // classic TIFF while the file stays below 4 GB (as GDAL's BIGTIFF=IF_NEEDED
    // decides for uncompressed data), BigTIFF beyond, or when asked
    const bool big = force_bigtiff || total > 0xF0000000ull;
    const uint32_t per = (uint32_t)std::max<size_t>(1, std::min<size_t>(m.rows, 65536 / std::max<size_t>(rowbytes, 1)));
    const uint32_t nstrips = (uint32_t)((m.rows + per - 1) / per);
    Writer w;
    w.u32(256, (uint32_t)m.cols);
    w.u32(257, (uint32_t)m.rows);
    w.u16(258, (uint16_t)(bpp * 8));
    w.u16(259, 1);
    w.u16(262, 1);
    // strip offsets (patched below) and byte counts: LONG, or LONG8 in BigTIFF
    const size_t osz = big ? 8 : 4;
    std::vector<unsigned char> offs(osz * nstrips, 0), counts(osz * nstrips, 0);
    for (uint32_t s = 0; s < nstrips; s++) {
        const uint64_t c = std::min<uint64_t>(per, m.rows - (uint64_t)s * per) * rowbytes;
        if (big) memcpy(counts.data() + 8 * (size_t)s, &c, 8);
        else {
            const uint32_t c32 = (uint32_t)c;
            memcpy(counts.data() + 4 * (size_t)s, &c32, 4);
        }
    }
    const size_t i_offs = w.entries.size();
    w.add(273, big ? 16 : 4, nstrips, offs.data(), offs.size());
    w.u16(277, 1);
    w.u32(278, per);
    w.add(279, big ? 16 : 4, nstrips, counts.data(), counts.size());
    w.u16(284, 1);
    w.u16(339, 3);
    const double scale[3] = {m.transform[1], -m.transform[5], 0.0};
    const double tie[6] = {0.0, 0.0, 0.0, m.transform[0], m.transform[3], 0.0};
    w.add(33550, 12, 3, scale, sizeof(scale));
    w.add(33922, 12, 6, tie, sizeof(tie));
    if (!m.geokeys.empty()) w.add(34735, 3, m.geokeys.size() / 2, m.geokeys.data(), m.geokeys.size());
    if (!m.geodoubles.empty()) w.add(34736, 12, m.geodoubles.size() / 8, m.geodoubles.data(), m.geodoubles.size());
    if (!m.geoascii.empty()) w.add(34737, 2, m.geoascii.size(), m.geoascii.data(), m.geoascii.size());
    char nd[64];
    snprintf(nd, sizeof(nd), "%.17g", m.nodata);
    std::string nds(nd);
    nds.push_back('\0');
    w.add(42113, 2, nds.size(), nds.data(), nds.size());
    // layout: header, IFD, out-of-line values, strips
    const size_t n = w.entries.size();
    const size_t inline_max = big ? 8 : 4;
    const size_t ifd_off = big ? 16 : 8, ifd_size = big ? 8 + 20 * n + 8 : 2 + 12 * n + 4;
    size_t cursor = ifd_off + ifd_size;
    std::vector<size_t> value_off(n, 0);
    for (size_t i = 0; i < n; i++) {
        if (w.entries[i].data.size() > inline_max) {
            value_off[i] = cursor;
            cursor += (w.entries[i].data.size() + 1) & ~(size_t)1;
        }
    }
    const size_t data_off = (cursor + 15) & ~(size_t)15;
    for (uint32_t s = 0; s < nstrips; s++) {
        const uint64_t o = data_off + (uint64_t)s * per * rowbytes;
        if (big) memcpy(w.entries[i_offs].data.data() + 8 * (size_t)s, &o, 8);
        else {
            const uint32_t o32 = (uint32_t)o;
            memcpy(w.entries[i_offs].data.data() + 4 * (size_t)s, &o32, 4);
        }
    }
    std::vector<unsigned char> out;  // header, IFD and tag values; the samples are streamed after them
    out.reserve(data_off);
    out.push_back('I');
    out.push_back('I');
    if (big) {
        put16(out, 43);
        put16(out, 8);
        put16(out, 0);
        put64(out, ifd_off);
        put64(out, n);
    } else {
        put16(out, 42);
        put32(out, (uint32_t)ifd_off);
        put16(out, (uint16_t)n);
    }
    for (size_t i = 0; i < n; i++) {
        const auto& e = w.entries[i];
        put16(out, e.tag);
        put16(out, e.type);
        if (big) put64(out, e.count);
        else put32(out, (uint32_t)e.count);
        if (e.data.size() > inline_max) {
            if (big) put64(out, value_off[i]);
            else put32(out, (uint32_t)value_off[i]);
        } else {
            unsigned char v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            memcpy(v, e.data.data(), e.data.size());
            out.insert(out.end(), v, v + inline_max);
        }
    }
    if (big) put64(out, 0);
    else put32(out, 0);
    for (size_t i = 0; i < n; i++) {
        const auto& e = w.entries[i];
        if (e.data.size() > inline_max) {
            out.insert(out.end(), e.data.begin(), e.data.end());
            if (e.data.size() & 1) out.push_back(0);
        }
    }
    out.resize(data_off, 0);
    std::ofstream f(path, std::ios::binary);
    if (!f) {
        *err = std::string("cannot create ") + path;
        return false;
    }
    f.write((const char*)out.data(), (std::streamsize)out.size());
    // the samples, little-endian, through a buffer of about 4 MB
    const size_t n_all = (size_t)m.rows * m.cols, chunk = (size_t)1 << 19;
    std::vector<unsigned char> buf(chunk * bpp);
    for (size_t i0 = 0; i0 < n_all && f; i0 += chunk) {
        const size_t k_n = std::min(chunk, n_all - i0);
        if (bpp == 4) {
            for (size_t k = 0; k < k_n; k++) {
                const float v = (float)values[i0 + k];
                memcpy(buf.data() + 4 * k, &v, 4);
            }
        } else {
            memcpy(buf.data(), values + i0, 8 * k_n);
        }
        f.write((const char*)buf.data(), (std::streamsize)(k_n * bpp));
    }
    if (!f) *err = std::string(path) + ": write failed";
    return (bool)f;
}

}  // namespace GPRO
