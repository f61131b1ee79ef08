// lb_case.cu -- case files (include/lbgb300.h, parts 5 and 6): the parameter
// (.dat) and bitmap (.bmp) readers of the reference's Input class
// (src/input.cpp:51-116), the initial states its Simulation constructors
// build (src/simulation_d2q9.cu:100-334, src/simulation_d3q19.cu:99-204) and
// the VTK files of its Output class (src/output.cpp:52-155).
//
// Host code only.  The initial states are bit-identical to the reference's:
// every float and double operation is written in the reference's order and
// type (float products, FP64 promotions by the double literals), and the
// library's host code is compiled without floating-point contraction.
#include <charconv>
#include <cfloat>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/lbgb300.h"
#include "lb_kernels.cuh"

namespace {

int fail(int code, const char *where, const std::string &what) {
    lb::abi_record_error(where, what.c_str());
    return code;
}

// ---------------------------------------------------------------- .dat file

// one line as a Qt text stream returns it: without "\n" or "\r\n"; an empty
// line past the end of the file
void read_line(FILE *fp, std::string &line) {
    line.clear();
    int ch;
    while ((ch = std::fgetc(fp)) != EOF && ch != '\n') line.push_back((char)ch);
    if (!line.empty() && line.back() == '\r') line.pop_back();
}

bool is_space(char c) {
    return c == ' ' || c == '\t' || c == '\n' || c == '\v' || c == '\f' || c == '\r';
}

std::string trimmed(const std::string &s) {
    size_t a = 0, b = s.size();
    while (a < b && is_space(s[a])) a++;
    while (b > a && is_space(s[b - 1])) b--;
    return s.substr(a, b - a);
}

// QString::toInt semantics: surrounding white space allowed, an optional sign,
// decimal digits only; anything else, or a value outside int, reads as 0
int to_int(const std::string &line) {
    const std::string t = trimmed(line);
    if (t.empty()) return 0;
    size_t i = (t[0] == '+' || t[0] == '-') ? 1 : 0;
    if (i == t.size()) return 0;
    long long v = 0;
    for (size_t j = i; j < t.size(); j++) {
        if (t[j] < '0' || t[j] > '9') return 0;
        v = v * 10 + (t[j] - '0');
        if (v > 2147483648LL) return 0;
    }
    if (t[0] == '-') v = -v;
    if (v > 2147483647LL || v < -2147483648LL) return 0;
    return (int)v;
}

// QString::toFloat semantics: the C-locale decimal syntax (optional sign,
// digits with an optional point, optional exponent; "inf"/"nan"), rounded to
// double and then to float; a finite value beyond the float range, or a
// string that is not a number, reads as 0
float to_float(const std::string &line) {
    std::string t = trimmed(line);
    if (t.empty()) return 0.f;
    std::string low;
    for (char c : t) low.push_back((c >= 'A' && c <= 'Z') ? (char)(c - 'A' + 'a') : c);
    const char *s = low.c_str();
    bool neg = false;
    if (*s == '+' || *s == '-') { neg = *s == '-'; s++; }
    if (!std::strcmp(s, "inf") || !std::strcmp(s, "infinity")) return neg ? -INFINITY : INFINITY;
    if (!std::strcmp(s, "nan")) return NAN;
    // the grammar check: from_chars alone would also take hex digits
    const char *q = s;
    bool digits = false;
    while (*q >= '0' && *q <= '9') { q++; digits = true; }
    if (*q == '.') {
        q++;
        while (*q >= '0' && *q <= '9') { q++; digits = true; }
    }
    if (!digits) return 0.f;
    if (*q == 'e') {
        q++;
        if (*q == '+' || *q == '-') q++;
        if (!(*q >= '0' && *q <= '9')) return 0.f;
        while (*q >= '0' && *q <= '9') q++;
    }
    if (*q != '\0') return 0.f;
    double d = 0.0;
    const auto r = std::from_chars(s, q, d, std::chars_format::general);
    if (r.ec == std::errc::result_out_of_range) {
        // overflow reads as 0 (beyond float anyway); underflow rounds to 0
        return 0.f;
    }
    if (r.ec != std::errc() || r.ptr != q) return 0.f;
    if (neg) d = -d;
    if (std::fabs(d) > (double)FLT_MAX) return 0.f;
    return (float)d;
}

// ---------------------------------------------------------------- .bmp file

uint32_t rd16(const uint8_t *p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
uint32_t rd32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) |
           ((uint32_t)p[3] << 24);
}

struct Bitmap {
    int width = 0, height = 0;
    bool top_down = false;
    int bpp = 0;
    uint32_t rmask = 0, gmask = 0, bmask = 0, amask = 0;
    std::vector<uint8_t> black;  // palette images: 1 where the entry is black
    size_t data_off = 0, stride = 0;
};

bool read_file(const char *path, std::vector<uint8_t> &bytes) {
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return false;
    bytes.clear();
    uint8_t buf[65536];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) bytes.insert(bytes.end(), buf, buf + n);
    const bool ok = !std::ferror(fp);
    std::fclose(fp);
    return ok;
}

// parse the headers; "" on success, else what is wrong
std::string parse_bmp(const std::vector<uint8_t> &b, Bitmap &bm) {
    if (b.size() < 26 || b[0] != 'B' || b[1] != 'M') return "not a Windows bitmap";
    const uint32_t off_bits = rd32(&b[10]);
    const uint32_t hsize = rd32(&b[14]);
    uint32_t compression = 0, clr_used = 0;
    int64_t w, h;
    size_t pal_entry = 4;
    if (hsize == 12) {  // BITMAPCOREHEADER
        w = rd16(&b[18]);
        h = (int16_t)rd16(&b[20]);
        bm.bpp = (int)rd16(&b[24]);
        pal_entry = 3;
    } else if (hsize >= 40 && hsize <= 124) {
        if (b.size() < 14 + (size_t)hsize) return "truncated header";
        w = (int32_t)rd32(&b[18]);
        h = (int32_t)rd32(&b[22]);
        bm.bpp = (int)rd16(&b[28]);
        compression = rd32(&b[30]);
        clr_used = rd32(&b[46]);
    } else {
        return "unsupported header size " + std::to_string(hsize);
    }
    if (w <= 0 || h == 0) return "bad image size";
    bm.top_down = h < 0;
    if (h < 0) h = -h;
    if (w > (1 << 20) || h > (1 << 20) || w * h > (int64_t)1 << 30) return "image too large";
    bm.width = (int)w;
    bm.height = (int)h;
    const int bpp = bm.bpp;
    if (bpp != 1 && bpp != 4 && bpp != 8 && bpp != 16 && bpp != 24 && bpp != 32)
        return "unsupported bits per pixel " + std::to_string(bpp);
    if (compression == 3) {  // BI_BITFIELDS
        if (bpp != 16 && bpp != 32) return "BI_BITFIELDS needs 16 or 32 bits per pixel";
        size_t mo = 14 + 40;  // masks follow a 40-byte header, or sit inside a longer one
        if (b.size() < mo + 12) return "truncated header";
        bm.rmask = rd32(&b[mo]);
        bm.gmask = rd32(&b[mo + 4]);
        bm.bmask = rd32(&b[mo + 8]);
        if (hsize >= 56) bm.amask = rd32(&b[mo + 12]);
    } else if (compression == 0) {
        if (bpp == 16) { bm.rmask = 0x7c00; bm.gmask = 0x03e0; bm.bmask = 0x001f; }
        if (bpp == 32) { bm.rmask = 0xff0000; bm.gmask = 0xff00; bm.bmask = 0xff; }
    } else {
        return "unsupported compression " + std::to_string(compression);
    }
    if (bpp <= 8) {
        size_t ncol = clr_used ? clr_used : (1u << bpp);
        if (ncol > 256) return "bad colour table size";
        size_t po = 14 + hsize;
        if (b.size() < po + ncol * pal_entry) return "truncated colour table";
        bm.black.assign(ncol, 0);
        for (size_t i = 0; i < ncol; i++) {
            const uint8_t *e = &b[po + i * pal_entry];  // blue, green, red[, reserved]
            bm.black[i] = (e[0] == 0 && e[1] == 0 && e[2] == 0) ? 1 : 0;
        }
    }
    bm.stride = (((size_t)bm.width * bpp + 31) / 32) * 4;
    bm.data_off = off_bits;
    if (bm.data_off > b.size() || b.size() - bm.data_off < bm.stride * (size_t)bm.height)
        return "truncated pixel data";
    return "";
}

// is pixel (x, row r of the file) opaque black
bool pixel_black(const Bitmap &bm, const uint8_t *row, int x) {
    switch (bm.bpp) {
        case 1:
        case 4:
        case 8: {
            const int per = 8 / bm.bpp;
            const uint8_t byte = row[x / per];
            const int shift = 8 - bm.bpp * (x % per + 1);
            const unsigned idx = (byte >> shift) & ((1u << bm.bpp) - 1);
            // an index past the colour table is not black
            return idx < bm.black.size() && bm.black[idx];
        }
        case 24: {
            const uint8_t *p = row + 3 * (size_t)x;
            return p[0] == 0 && p[1] == 0 && p[2] == 0;
        }
        default: {
            const uint32_t v = bm.bpp == 16 ? rd16(row + 2 * (size_t)x) : rd32(row + 4 * (size_t)x);
            if ((v & bm.rmask) || (v & bm.gmask) || (v & bm.bmask)) return false;
            return !bm.amask || (v & bm.amask) == bm.amask;
        }
    }
}

// ------------------------------------------------------------- initial state

// f_eq of the reference host code: w*rho in float, the bracket in double
// (1. + 3.*s + 4.5*s*s - 1.5*usq with s a float), the product rounded to float
inline float feq_ref(float w, float rho, float s, float usq) {
    const float wr = w * rho;
    return (float)((double)wr * (((1. + 3. * (double)s) + (4.5 * (double)s) * (double)s) -
                                 1.5 * (double)usq));
}
inline float feq0_ref(float w, float rho, float usq) {
    const float wr = w * rho;
    return (float)((double)wr * (1. - 1.5 * (double)usq));
}

}  // namespace

extern "C" {

int lb_case_load_parameters(const char *path, lb_case_params *out) {
    if (!path || !out) return fail(LB_ERR_ARG, "lb_case_load_parameters", "null argument");
    FILE *fp = std::fopen(path, "rb");
    if (!fp) return fail(LB_ERR_IO, "lb_case_load_parameters", std::string("cannot open ") + path);
    std::string line;
    lb_case_params p;
    std::memset(&p, 0, sizeof p);
    read_line(fp, line); p.device_count = to_int(line);
    read_line(fp, line); p.max_dim = to_int(line);
    if (p.max_dim < 2) p.max_dim = 1;  // src/input.cpp:149-152
    read_line(fp, line); p.ux = to_float(line);
    read_line(fp, line); p.uy = to_float(line);
    read_line(fp, line); p.uz = to_float(line);
    read_line(fp, line); p.rho = to_float(line);
    read_line(fp, line); p.viscosity = to_float(line);
    p.tau_inv = (float)(1. / (3. * (double)p.viscosity + 0.5));
    read_line(fp, line); p.update_steps = to_int(line);
    for (int i = 0; i < 3; i++) { read_line(fp, line); p.ext_f[i] = to_float(line); }
    read_line(fp, line); p.G = to_float(line);
    read_line(fp, line); p.G_ads = to_float(line);
    const bool err = std::ferror(fp) != 0;
    std::fclose(fp);
    if (err) return fail(LB_ERR_IO, "lb_case_load_parameters", std::string("read error in ") + path);
    p.min_u = 0.0f;
    p.max_u = (float)((double)p.ux * 1.5);
    p.min_rho = (float)((double)p.rho * 0.98);
    p.max_rho = (float)((double)p.rho * 1.02);
    *out = p;
    return LB_OK;
}

int lb_case_load_solids_bmp(const char *path, int *width, int *height, uint8_t *solids,
                            size_t capacity) {
    const char *where = "lb_case_load_solids_bmp";
    if (!path || !width || !height) return fail(LB_ERR_ARG, where, "null argument");
    std::vector<uint8_t> b;
    if (!read_file(path, b)) return fail(LB_ERR_IO, where, std::string("cannot read ") + path);
    Bitmap bm;
    const std::string why = parse_bmp(b, bm);
    if (!why.empty()) return fail(LB_ERR_IO, where, std::string(path) + ": " + why);
    *width = bm.width;
    *height = bm.height;
    if (!solids) return LB_OK;
    const size_t n = (size_t)bm.width * bm.height;
    if (capacity < n) return fail(LB_ERR_ARG, where, "solids buffer too small");
    for (int y = 0; y < bm.height; y++) {
        // y = 0 is the top row: the last row stored in a bottom-up file
        const int r = bm.top_down ? y : bm.height - 1 - y;
        const uint8_t *row = &b[bm.data_off + (size_t)r * bm.stride];
        for (int x = 0; x < bm.width; x++)
            solids[(size_t)y * bm.width + x] = pixel_black(bm, row, x) ? 1 : 0;
    }
    return LB_OK;
}

int lb_case_init_d2q9(const lb_case_params *p, int W, int H, const uint8_t *solids, float *f,
                      float *ux, float *uy, float *rho, float *psi_out, float *ueq_x_out,
                      float *ueq_y_out, uint8_t *solid_bound) {
    const char *where = "lb_case_init_d2q9";
    if (!p || !solids || !f || !ux || !uy || !rho || !solid_bound)
        return fail(LB_ERR_ARG, where, "null argument");
    if (W < 1 || H < 1 || (int64_t)W * H > (int64_t)1 << 30)
        return fail(LB_ERR_ARG, where, "bad extents");
    const long N = (long)W * H;
    std::vector<float> psi_v, ueqx_v, ueqy_v;
    float *psi = psi_out, *ueq_x = ueq_x_out, *ueq_y = ueq_y_out;
    if (!psi) { psi_v.assign(N, 0.f); psi = psi_v.data(); }
    if (!ueq_x) { ueqx_v.assign(N, 0.f); ueq_x = ueqx_v.data(); }
    if (!ueq_y) { ueqy_v.assign(N, 0.f); ueq_y = ueqy_v.data(); }
    float *fk[9];
    for (int k = 0; k < 9; k++) fk[k] = f + (long)k * N;
    for (long i = 0; i < N; i++) {
        ux[i] = uy[i] = rho[i] = psi[i] = ueq_x[i] = ueq_y[i] = 0.f;
        for (int k = 0; k < 9; k++) fk[k][i] = 0.f;
        solid_bound[i] = 0;
    }
    // the weights of src/simulation_d2q9.cu:51-53, as float members
    const float w0 = (float)(16. / 36.), w1 = (float)(4. / 36.), w2 = (float)(1. / 36.);
    ux[0] = p->ux;
    uy[0] = p->uy;
    rho[0] = p->rho;
    ueq_x[0] = p->ux;
    ueq_y[0] = p->uy;
    float tauInv = 0.f;
    if (p->ext_f[0] != 0) {
        tauInv = p->tau_inv;
        ueq_x[0] = ux[0] + p->ext_f[0] / (tauInv * rho[0]);
    }
    if (p->ext_f[1] != 0) {
        tauInv = p->tau_inv;
        ueq_y[0] = uy[0] + p->ext_f[1] / (tauInv * rho[0]);
    }
    auto feq_all = [&](long o, float r, float ex, float ey) {
        const float usq = ex * ex + ey * ey;
        fk[0][o] = feq0_ref(w0, r, usq);
        fk[1][o] = feq_ref(w1, r, +ex, usq);
        fk[2][o] = feq_ref(w1, r, +ey, usq);
        fk[3][o] = feq_ref(w1, r, -ex, usq);
        fk[4][o] = feq_ref(w1, r, -ey, usq);
        fk[5][o] = feq_ref(w2, r, ex + ey, usq);
        fk[6][o] = feq_ref(w2, r, -ex + ey, usq);
        fk[7][o] = feq_ref(w2, r, -ex - ey, usq);
        fk[8][o] = feq_ref(w2, r, ex - ey, usq);
    };
    if (p->G != 0) {
        // Shan-Chen start (src/simulation_d2q9.cu:123-255): uniform density on
        // the fluid nodes, psi = 4 exp(-200/rho) in FP64, u_eq shifted by the
        // interaction and adhesion forces, forced equilibrium
        const float G = p->G, Gads = p->G_ads;
        tauInv = p->tau_inv;
        const float rho_aux = p->rho;
        for (int y = 0; y < H; y++)
            for (int x = 0; x < W; x++) {
                const long o = (long)y * W + x;
                if (solids[o]) continue;
                rho[o] = rho_aux;
                psi[o] = (float)(4. * std::exp(-200. / (double)rho[o]));
                ux[o] = ux[0];
                uy[o] = uy[0];
            }
        for (int y = 0; y < H; y++) {
            const int yp = (y < H - 1) ? y + 1 : 0;
            const int yn = (y > 0) ? y - 1 : H - 1;
            for (int x = 0; x < W; x++) {
                const int xp = (x < W - 1) ? x + 1 : 0;
                const int xn = (x > 0) ? x - 1 : W - 1;
                const long o = (long)y * W + x;
                if (solids[o]) continue;
                const long o1 = (long)y * W + xp, o2 = (long)yp * W + x, o3 = (long)y * W + xn,
                           o4 = (long)yn * W + x, o5 = (long)yp * W + xp, o6 = (long)yp * W + xn,
                           o7 = (long)yn * W + xn, o8 = (long)yn * W + xp;
                float IFx = 0, IFy = 0;
                IFx = IFx + w1 * psi[o1];
                IFx = IFx - w1 * psi[o3];
                IFx = IFx + w2 * psi[o5];
                IFx = IFx - w2 * psi[o6];
                IFx = IFx - w2 * psi[o7];
                IFx = IFx + w2 * psi[o8];
                IFy = IFy + w1 * psi[o2];
                IFy = IFy - w1 * psi[o4];
                IFy = IFy + w2 * psi[o5];
                IFy = IFy + w2 * psi[o6];
                IFy = IFy - w2 * psi[o7];
                IFy = IFy - w2 * psi[o8];
                IFx = -G * psi[o] * IFx;
                IFy = -G * psi[o] * IFy;
                // node 0's u_eq is the base of every later node, and node 0
                // itself (when fluid) updates it first: the reference reads
                // ueq_x[0] live, so the same order is kept here
                ueq_x[o] = ueq_x[0] + (IFx / (tauInv * rho[o]));
                ueq_y[o] = ueq_y[0] + (IFy / (tauInv * rho[o]));
                float Fsx = 0, Fsy = 0;
                if (solids[o1]) Fsx = Fsx + w1;
                if (solids[o2]) Fsy = Fsy - w1;
                if (solids[o3]) Fsx = Fsx - w1;
                if (solids[o4]) Fsy = Fsy + w1;
                if (solids[o5]) { Fsx = Fsx + w2; Fsy = Fsy - w2; }
                if (solids[o6]) { Fsx = Fsx - w2; Fsy = Fsy - w2; }
                if (solids[o7]) { Fsx = Fsx - w2; Fsy = Fsy + w2; }
                if (solids[o8]) { Fsx = Fsx + w2; Fsy = Fsy + w2; }
                Fsx = -Gads * psi[o] * Fsx;
                Fsy = -Gads * psi[o] * Fsy;
                ueq_x[o] = ueq_x[o] + (Fsx / (tauInv * rho[o]));
                ueq_y[o] = ueq_y[o] + (Fsy / (tauInv * rho[o]));
                feq_all(o, rho[o], ueq_x[o], ueq_y[o]);
            }
        }
    } else {
        // uniform start (src/simulation_d2q9.cu:256-283), solid nodes included
        feq_all(0, rho[0], ueq_x[0], ueq_y[0]);
        for (long i = 1; i < N; i++) {
            ux[i] = ux[0];
            uy[i] = uy[0];
            rho[i] = rho[0];
            for (int k = 0; k < 9; k++) fk[k][i] = fk[k][0];
        }
    }
    // solid_bound (src/simulation_d2q9.cu:318-334): x in 1..W-2, periodic in y
    for (int y = 0; y < H; y++) {
        const int yn = (y > 0) ? y - 1 : H - 1;
        const int yp = (y < H - 1) ? y + 1 : 0;
        for (int x = 1; x < W - 1; x++) {
            const int xn = x - 1, xp = x + 1;
            auto s = [&](int xx, int yy) { return solids[(long)yy * W + xx] != 0; };
            solid_bound[(long)y * W + x] =
                (s(x, y) && s(xp, y) && s(x, yp) && s(xn, y) && s(x, yn) && s(xp, yp) &&
                 s(xn, yp) && s(xn, yn) && s(xp, yn)) ? 1 : 0;
        }
    }
    return LB_OK;
}

int lb_case_init_d3q19(const lb_case_params *p, int W, int H, int D, const uint8_t *solids,
                       float *f, float *ux, float *uy, float *uz, float *rho,
                       uint8_t *solid_bound) {
    const char *where = "lb_case_init_d3q19";
    if (!p || !solids || !f || !ux || !uy || !uz || !rho || !solid_bound)
        return fail(LB_ERR_ARG, where, "null argument");
    if (W < 1 || H < 1 || D < 1 || (int64_t)W * H * D > (int64_t)1 << 31)
        return fail(LB_ERR_ARG, where, "bad extents");
    const long N = (long)W * H * D;
    // the weights of src/simulation_d3q19.cu:54-56, as float members
    const float w0 = (float)(12. / 36.), w1 = (float)(2. / 36.), w2 = (float)(1. / 36.);
    const float x0 = p->ux, y0 = p->uy, z0 = p->uz, r0 = p->rho;
    const float usq = x0 * x0 + y0 * y0 + z0 * z0;
    float f0[19];
    f0[0] = feq0_ref(w0, r0, usq);
    f0[1] = feq_ref(w1, r0, +x0, usq);
    f0[2] = feq_ref(w1, r0, -x0, usq);
    f0[3] = feq_ref(w1, r0, +y0, usq);
    f0[4] = feq_ref(w1, r0, -y0, usq);
    f0[5] = feq_ref(w1, r0, +z0, usq);
    f0[6] = feq_ref(w1, r0, -z0, usq);
    f0[7] = feq_ref(w2, r0, +x0 + y0, usq);
    f0[8] = feq_ref(w2, r0, +x0 - y0, usq);
    f0[9] = feq_ref(w2, r0, +x0 + z0, usq);
    f0[10] = feq_ref(w2, r0, +x0 - z0, usq);
    f0[11] = feq_ref(w2, r0, -x0 + y0, usq);
    f0[12] = feq_ref(w2, r0, -x0 - y0, usq);
    f0[13] = feq_ref(w2, r0, -x0 + z0, usq);
    f0[14] = feq_ref(w2, r0, -x0 - z0, usq);
    f0[15] = feq_ref(w2, r0, +y0 + z0, usq);
    f0[16] = feq_ref(w2, r0, +y0 - z0, usq);
    f0[17] = feq_ref(w2, r0, -y0 + z0, usq);
    f0[18] = feq_ref(w2, r0, -y0 - z0, usq);
    for (long i = 0; i < N; i++) {
        ux[i] = x0;
        uy[i] = y0;
        uz[i] = i == 0 ? z0 : 0.f;  // the reference's fill loop skips uz
        rho[i] = r0;
        for (int k = 0; k < 19; k++) f[(long)k * N + i] = f0[k];
        solid_bound[i] = 0;
    }
    // solid_bound (src/simulation_d3q19.cu:167-204): x in 1..W-2, the node
    // and its 18 neighbours solid, periodic in y and z
    for (int z = 0; z < D; z++) {
        const int zn = (z > 0) ? z - 1 : D - 1, zp = (z < D - 1) ? z + 1 : 0;
        for (int y = 0; y < H; y++) {
            const int yn = (y > 0) ? y - 1 : H - 1, yp = (y < H - 1) ? y + 1 : 0;
            for (int x = 1; x < W - 1; x++) {
                const int xn = x - 1, xp = x + 1;
                auto s = [&](int xx, int yy, int zz) {
                    return solids[xx + (long)W * (yy + (long)H * zz)] != 0;
                };
                const bool all =
                    s(x, y, z) && s(xp, y, z) && s(xn, y, z) && s(x, yp, z) && s(x, yn, z) &&
                    s(x, y, zp) && s(x, y, zn) && s(xp, yp, z) && s(xp, yn, z) && s(xp, y, zp) &&
                    s(xp, y, zn) && s(xn, yp, z) && s(xn, yn, z) && s(xn, y, zp) &&
                    s(xn, y, zn) && s(x, yp, zp) && s(x, yp, zn) && s(x, yn, zp) && s(x, yn, zn);
                solid_bound[x + (long)W * (y + (long)H * z)] = all ? 1 : 0;
            }
        }
    }
    return LB_OK;
}

}  // extern "C"

// -------------------------------------------------------------------- VTK

namespace {

std::string join(const char *dir, const std::string &name) {
    if (!dir || !*dir) return name;
    std::string d(dir);
    if (d.back() != '/') d.push_back('/');
    return d + name;
}

// a float as an ostream with default settings prints it: "%g" of the value
// widened to double, 6 significant digits
inline void put_float(std::string &out, float v) {
    char buf[32];
    const int n = std::snprintf(buf, sizeof buf, "%g", (double)v);
    out.append(buf, (size_t)n);
}

bool write_all(const std::string &path, const std::string &text) {
    FILE *fp = std::fopen(path.c_str(), "wb");
    if (!fp) return false;
    const bool ok = std::fwrite(text.data(), 1, text.size(), fp) == text.size();
    return (std::fclose(fp) == 0) && ok;
}

std::string extent(int x0, int x1, int height, int length) {
    return std::to_string(x0) + " " + std::to_string(x1) + " 0 " + std::to_string(height - 1) +
           " 0 " + std::to_string(length - 1);
}

}  // namespace

extern "C" {

int lb_vtk_save(const char *dir, int vtk_id, int device_id, int width, int height, int length,
                const float *rho, const float *ux, const float *uy, const float *uz) {
    const char *where = "lb_vtk_save";
    if (vtk_id < 0 || vtk_id > 9999 || device_id < 0 || device_id > 99)
        return fail(LB_ERR_ARG, where, "vtk_id must be 0..9999 and device_id 0..99");
    if (width < 1 || height < 1 || length < 1 || !rho || !ux || !uy || (length > 1 && !uz))
        return fail(LB_ERR_ARG, where, "bad extents or null field");
    char name[32];
    std::snprintf(name, sizeof name, "r%04dp%02d.vti", vtk_id, device_id);
    const std::string ext = extent(device_id * width, (device_id + 1) * width, height, length);
    const long n = (long)width * height * length;
    std::string out;
    out.reserve((size_t)n * 48 + 1024);
    out += "<VTKFile type=\"ImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    out += "  <ImageData WholeExtent=\"" + ext + "\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n";
    out += "  <Piece Extent=\"" + ext + "\">\n";
    out += "    <PointData Scalars=\"Pressure\" Vectors=\"Velocity\">\n";
    out += "      <DataArray type=\"Float32\" Name=\"Pressure\" format=\"ascii\" >\n      ";
    for (long i = 0; i < n; i++) {
        put_float(out, rho[i]);
        out += ' ';
        if ((i + 1) % width == 0) out += "0\n      ";  // the closing x = width point
    }
    out += "</DataArray>\n";
    out += "      <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" "
           "format=\"ascii\">\n      ";
    for (long i = 0; i < n; i++) {
        put_float(out, ux[i]);
        out += ' ';
        if (length > 1) {
            put_float(out, uy[i]);
            out += ' ';
            put_float(out, uz[i]);
            out += "   ";
        } else {
            put_float(out, -uy[i]);  // image rows grow downwards
            out += " 0   ";
        }
        if ((i + 1) % width == 0) out += "0 0 0\n      ";
    }
    out += "</DataArray>\n    </PointData>\n    <CellData>\n    </CellData>\n  </Piece>\n"
           "  </ImageData>\n</VTKFile>\n";
    const std::string path = join(dir, name);
    if (!write_all(path, out)) return fail(LB_ERR_IO, where, "cannot write " + path);
    return LB_OK;
}

int lb_vtk_save_parallel(const char *dir, int vtk_id, int device_count, int width, int height,
                         int length) {
    const char *where = "lb_vtk_save_parallel";
    if (vtk_id < 0 || vtk_id > 9999 || device_count < 1 || device_count > 100)
        return fail(LB_ERR_ARG, where, "vtk_id must be 0..9999 and device_count 1..100");
    if (width < 1 || height < 1 || length < 1) return fail(LB_ERR_ARG, where, "bad extents");
    char name[32];
    std::snprintf(name, sizeof name, "r%04d.pvti", vtk_id);
    std::string out;
    out += "<VTKFile type=\"PImageData\" version=\"0.1\" byte_order=\"LittleEndian\">\n";
    out += "  <PImageData WholeExtent=\"" + extent(0, width * device_count - 1, height, length) +
           "\" GhostLevel=\"#\" Origin=\"0 0 0\" Spacing=\"1 1 1\">\n";
    out += "    <PPointData Scalars=\"Pressure\" Vectors=\"Velocity\">\n";
    out += "      <DataArray type=\"Float32\" Name=\"Pressure\" format=\"ascii\"/>\n";
    out += "      <DataArray type=\"Float32\" Name=\"Velocity\" NumberOfComponents=\"3\" "
           "format=\"ascii\"/>\n    </PPointData>\n    <PCellData>\n    </PCellData>\n";
    for (int i = 0; i < device_count; i++) {
        char piece[32];
        std::snprintf(piece, sizeof piece, "r%04dp%02d.vti", vtk_id, i);
        out += "    <Piece Extent=\"" + extent(i * width, (i + 1) * width, height, length) +
               "\" Source=\"" + piece + "\"/>\n";
    }
    out += "  </PImageData>\n</VTKFile>\n";
    const std::string path = join(dir, name);
    if (!write_all(path, out)) return fail(LB_ERR_IO, where, "cannot write " + path);
    return LB_OK;
}

}  // extern "C"
