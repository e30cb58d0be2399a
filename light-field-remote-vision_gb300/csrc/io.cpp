// io.cpp -- reference config files and PFM images.
//
// Config syntax of coco::config::parse_config_file (cocolib/cocolib/common/parse_config.cpp:44-101):
// each line "name value..." sets switch `name` to the text from the first occurrence of the value token to
// the end of the line; lines whose name starts with '#' are skipped; "config <file>" parses another file
// at that point (:179-181), so later lines override earlier ones. Config_data::parse_config
// (sources/config.cpp:67-129) then reads the solver keys and divides sigma_sensor by 255.
#include "lfrv.h"
#include "lfrv_internal.h"

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace {

std::mutex g_cfg_mutex;
std::map<std::string, std::string> g_switches;  // switches of the last parsed file

bool parse_file(const std::string &path, std::map<std::string, std::string> &sw, int depth) {
    if (depth > 32) return false;
    FILE *f = std::fopen(path.c_str(), "r");
    if (!f) return false;
    char line[600];
    bool ok = true;
    while (std::fgets(line, 500, f)) {
        size_t L = std::strlen(line);
        if (L > 0 && line[L - 1] == '\n') line[--L] = 0;
        char name[600], value[600];
        const int count = std::sscanf(line, "%599s %599s", name, value);
        if (count <= 0) continue;
        if (name[0] == '#') continue;
        if (count < 2) continue;  // a bare string (coco::config::add_string) sets no switch
        const char *loc = std::strstr(line + std::strlen(name), value);
        std::string sval = loc ? std::string(loc) : std::string(value);
        const std::string sname(name);
        if (sname == "config") ok = parse_file(sval, sw, depth + 1) && ok;
        sw[sname] = sval;
    }
    std::fclose(f);
    return ok;
}

// Numeric switches are read with sscanf semantics (leading number, trailing text ignored).
void get_int(const std::map<std::string, std::string> &sw, const char *k, int &v) {
    auto it = sw.find(k);
    if (it != sw.end()) v = std::atoi(it->second.c_str());
}
void get_float(const std::map<std::string, std::string> &sw, const char *k, float &v) {
    auto it = sw.find(k);
    if (it != sw.end()) v = (float)std::atof(it->second.c_str());
}

void apply_switches(const std::map<std::string, std::string> &sw, lfrv_config *cfg) {
    get_int(sw, "dsf", cfg->dsf);
    get_int(sw, "width", cfg->w);
    get_int(sw, "height", cfg->h);
    get_int(sw, "nchannels", cfg->nchannels);
    get_float(sw, "ugrad_threshold", cfg->ugrad_threshold);
    get_float(sw, "sigma_sensor", cfg->sigma_sensor);
    cfg->sigma_sensor = (float)(cfg->sigma_sensor / 255.0);  // sources/config.cpp:119, applied unconditionally
    get_float(sw, "lambda", cfg->lambda);
    get_float(sw, "lambda_max_factor", cfg->lambda_max_factor);
    get_int(sw, "dw_type", cfg->dw_type);
    get_int(sw, "gw_type", cfg->gw_type);
    get_float(sw, "dt_alpha", cfg->dt_alpha);
    get_float(sw, "dt_beta", cfg->dt_beta);
    get_int(sw, "niter", cfg->niter);
    get_int(sw, "nmeta_iter", cfg->nmeta_iter);
    get_float(sw, "gradient_step", cfg->gradient_step);
    int s_min = -1, s_max = -1, s_rmv = -1;
    get_int(sw, "s_min", s_min);
    get_int(sw, "s_max", s_max);
    get_int(sw, "s_rmv", s_rmv);
    if (s_max >= s_min && s_min >= 0) cfg->nviews = (s_max - s_min + 1) - ((s_rmv >= s_min && s_rmv <= s_max) ? 1 : 0);
}

inline bool little_endian() {
    const uint16_t x = 1;
    return *(const uint8_t *)&x == 1;
}

void swap_bytes(float *p, size_t n) {
    for (size_t i = 0; i < n; ++i) {
        uint8_t *b = (uint8_t *)(p + i);
        std::swap(b[0], b[3]);
        std::swap(b[1], b[2]);
    }
}

}  // namespace

extern "C" int lfrv_config_default(lfrv_config *cfg) {
    if (!cfg) return lfrv::fail(LFRV_E_ARG, "null config");
    std::memset(cfg, 0, sizeof(*cfg));
    // Config_data::Config_data (sources/config.cpp:11-64)
    cfg->w = cfg->h = 0;
    cfg->dsf = 0;
    cfg->nviews = 0;
    cfg->nchannels = 0;
    cfg->sigma_sensor = (float)(1. / 255.0);
    cfg->ugrad_threshold = 1.0f;
    cfg->lambda = 0.0f;
    cfg->lambda_max_factor = 0.0f;
    cfg->dw_type = 0;
    cfg->gw_type = 0;
    cfg->dt_alpha = 1.0f;
    cfg->dt_beta = 0.0f;
    cfg->niter = 0;
    cfg->nmeta_iter = 1;
    cfg->gradient_step = 0.1f;
    // options of this library
    cfg->faithful = 1;
    cfg->early_exit = 1;
    cfg->cg_max_iter = 500;
    cfg->cg_gap_tol = 1e-4;
    cfg->hole_fill_iter = 500;
    cfg->bf16_storage = 0;
    return LFRV_OK;
}

extern "C" int lfrv_config_parse_file(const char *path, lfrv_config *cfg) {
    if (!path || !cfg) return lfrv::fail(LFRV_E_ARG, "null argument");
    std::map<std::string, std::string> sw;
    if (!parse_file(path, sw, 0)) return lfrv::fail(LFRV_E_IO, "could not read config file %s", path);
    apply_switches(sw, cfg);
    std::lock_guard<std::mutex> lock(g_cfg_mutex);
    g_switches = sw;
    return LFRV_OK;
}

extern "C" int lfrv_config_set(lfrv_config *cfg, const char *key, const char *value) {
    if (!cfg || !key || !value) return lfrv::fail(LFRV_E_ARG, "null argument");
    std::map<std::string, std::string> sw;
    sw[key] = value;
    const float sigma_before = cfg->sigma_sensor;
    apply_switches(sw, cfg);
    if (std::strcmp(key, "sigma_sensor") != 0) cfg->sigma_sensor = sigma_before;
    std::lock_guard<std::mutex> lock(g_cfg_mutex);
    g_switches[key] = value;
    return LFRV_OK;
}

extern "C" int lfrv_config_get_string(const char *key, char *buf, size_t buflen) {
    if (!key || !buf || buflen == 0) return lfrv::fail(LFRV_E_ARG, "null argument");
    std::lock_guard<std::mutex> lock(g_cfg_mutex);
    auto it = g_switches.find(key);
    if (it == g_switches.end()) return lfrv::fail(LFRV_E_ARG, "key %s not set", key);
    // values are the text after the key; trailing blanks are not part of a path
    std::string v = it->second;
    while (!v.empty() && (v.back() == ' ' || v.back() == '\t' || v.back() == '\r')) v.pop_back();
    std::snprintf(buf, buflen, "%s", v.c_str());
    return LFRV_OK;
}

extern "C" int lfrv_config_get_int(const char *key, int *value) {
    if (!key || !value) return lfrv::fail(LFRV_E_ARG, "null argument");
    std::lock_guard<std::mutex> lock(g_cfg_mutex);
    auto it = g_switches.find(key);
    if (it == g_switches.end()) return lfrv::fail(LFRV_E_ARG, "key %s not set", key);
    *value = std::atoi(it->second.c_str());
    return LFRV_OK;
}

// PFM reader following gsl_image_load_pfm (cocolib/cocolib/common/gsl_image.cpp:416-500): "PF" colour or
// "Pf" grey header, width/height line, scale line (negative = little endian), rows bottom-up.
extern "C" int lfrv_pfm_read(const char *path, int *w, int *h, int *channels, float *data, size_t capacity) {
    if (!path || !w || !h || !channels) return lfrv::fail(LFRV_E_ARG, "null argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return lfrv::fail(LFRV_E_IO, "cannot open %s", path);
    char type[3] = {0, 0, 0};
    int W = 0, H = 0;
    double scale = 0;
    auto bad = [&](const char *why) {
        std::fclose(f);
        return lfrv::fail(LFRV_E_FORMAT, "%s: %s", path, why);
    };
    if (std::fscanf(f, "%2s", type) != 1 || type[0] != 'P' || (type[1] != 'F' && type[1] != 'f'))
        return bad("PFM header not found");
    if (std::fscanf(f, "%d %d", &W, &H) != 2 || W <= 0 || H <= 0 || (long long)W * H > (1ll << 30))
        return bad("bad width/height");
    if (std::fscanf(f, "%lf", &scale) != 1) return bad("missing scale");
    std::fgetc(f);
    const int C = (type[1] == 'F') ? 3 : 1;
    *w = W;
    *h = H;
    *channels = C;
    if (!data) {
        std::fclose(f);
        return LFRV_OK;
    }
    const size_t N = (size_t)W * H;
    if (capacity < (size_t)C * N) {
        std::fclose(f);
        return lfrv::fail(LFRV_E_ARG, "%s: buffer holds %zu floats, need %zu", path, capacity, (size_t)C * N);
    }
    const bool invert = (scale > 0) == little_endian();  // scale > 0 marks big-endian data
    std::vector<float> row((size_t)C * W);
    for (int y = 0; y < H; ++y) {
        if (std::fread(row.data(), sizeof(float), row.size(), f) != row.size()) return bad("truncated data");
        if (invert) swap_bytes(row.data(), row.size());
        const int yy = H - 1 - y;  // rows are stored bottom-up
        for (int x = 0; x < W; ++x)
            for (int c = 0; c < C; ++c) data[(size_t)c * N + (size_t)yy * W + x] = row[(size_t)x * C + c];
    }
    std::fclose(f);
    return LFRV_OK;
}

// PFM writer following write_pfm_image_signed (cocolib/cocolib/cuda/cuda_helper.cu:340-375).
extern "C" int lfrv_pfm_write(const char *path, int w, int h, int channels, const float *data) {
    if (!path || !data || w <= 0 || h <= 0 || (channels != 1 && channels != 3))
        return lfrv::fail(LFRV_E_ARG, "bad arguments");
    FILE *f = std::fopen(path, "wb");
    if (!f) return lfrv::fail(LFRV_E_IO, "cannot create %s", path);
    std::fprintf(f, "P%c\n%d %d\n%d.0\n", channels == 3 ? 'F' : 'f', w, h, little_endian() ? -1 : 1);
    const size_t N = (size_t)w * h;
    std::vector<float> row((size_t)channels * w);
    for (int y = h - 1; y >= 0; --y) {
        for (int x = 0; x < w; ++x)
            for (int c = 0; c < channels; ++c) row[(size_t)x * channels + c] = data[(size_t)c * N + (size_t)y * w + x];
        if (std::fwrite(row.data(), sizeof(float), row.size(), f) != row.size()) {
            std::fclose(f);
            return lfrv::fail(LFRV_E_IO, "write failed: %s", path);
        }
    }
    std::fclose(f);
    return LFRV_OK;
}

// ------------------------------------------------------------------ MVE depth and normal maps
// InputView::importMVEIFile (sources/openGL/view.cpp:279-325): a text header line, then width, height, channels and
// type as four 32-bit unsigned integers, then height x width pixels of `channels` interleaved 32-bit floats (row 0
// first). Returned planar, top-left origin, like every other image here.
extern "C" int lfrv_mvei_read(const char *path, int *w, int *h, int *channels, float *data, size_t capacity) {
    if (!path || !w || !h || !channels) return lfrv::fail(LFRV_E_ARG, "null argument");
    FILE *f = std::fopen(path, "rb");
    if (!f) return lfrv::fail(LFRV_E_IO, "cannot open %s", path);
    auto bad = [&](const char *why) {
        std::fclose(f);
        return lfrv::fail(LFRV_E_FORMAT, "%s: %s", path, why);
    };
    int ch = 0;
    while ((ch = std::fgetc(f)) != EOF && ch != '\n') {
    }
    if (ch == EOF) return bad("MVEI header line not terminated");
    uint32_t hdr[4];
    if (std::fread(hdr, sizeof(uint32_t), 4, f) != 4) return bad("truncated size fields");
    if (!little_endian()) swap_bytes(reinterpret_cast<float *>(hdr), 4);
    const uint32_t W = hdr[0], H = hdr[1], C = hdr[2];
    if (W == 0 || H == 0 || C == 0 || C > 64 || (unsigned long long)W * H > (1ull << 30)) return bad("bad dimensions");
    *w = (int)W;
    *h = (int)H;
    *channels = (int)C;
    if (!data) {
        std::fclose(f);
        return LFRV_OK;
    }
    const size_t N = (size_t)W * H;
    if (capacity < (size_t)C * N) {
        std::fclose(f);
        return lfrv::fail(LFRV_E_ARG, "%s: buffer holds %zu floats, need %zu", path, capacity, (size_t)C * N);
    }
    std::vector<float> row((size_t)C * W);
    for (uint32_t y = 0; y < H; ++y) {
        if (std::fread(row.data(), sizeof(float), row.size(), f) != row.size()) return bad("truncated data");
        if (!little_endian()) swap_bytes(row.data(), row.size());
        for (uint32_t x = 0; x < W; ++x)
            for (uint32_t c = 0; c < C; ++c) data[(size_t)c * N + (size_t)y * W + x] = row[(size_t)x * C + c];
    }
    std::fclose(f);
    return LFRV_OK;
}

// InputView::setDepthAndNormals (sources/openGL/view.cpp:607-635) with Texture::loadFromData (sources/openGL/
// texture.cpp:207-290, no flip): the depth plane and the first two normal planes become the three depth-map channels,
// upsampled by nearest neighbour from (w0, h0) to (w0 * factor, h0 * factor); a pixel whose three values are all 0
// becomes (invalid_depth, 0, 0).
extern "C" int lfrv_depth_from_mve(int w0, int h0, int factor, const float *depth, const float *normal,
                                   float invalid_depth, float *out) {
    if (w0 <= 0 || h0 <= 0 || factor < 1 || !depth || !normal || !out) return lfrv::fail(LFRV_E_ARG, "bad arguments");
    const int W = w0 * factor, H = h0 * factor;
    const size_t n0 = (size_t)w0 * h0, N = (size_t)W * H;
    const float *src[3] = {depth, normal, normal + n0};
    for (int y = 0; y < H; ++y)
        for (int x = 0; x < W; ++x) {
            const size_t o = (size_t)y * W + x, s = (size_t)(y / factor) * w0 + (x / factor);
            const float a = src[0][s], b = src[1][s], c = src[2][s];
            const bool empty = a == 0.0f && b == 0.0f && c == 0.0f;
            out[o] = empty ? invalid_depth : a;
            out[N + o] = empty ? 0.0f : b;
            out[2 * N + o] = empty ? 0.0f : c;
        }
    return LFRV_OK;
}
