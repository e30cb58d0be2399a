// ulf_main.cpp -- config-driven command-line front end over liblfrv, for the IBR_color / IBR_gradient path.
//
// Usage mirrors the reference's executable (sources/main.cpp:56-443, coco::config::parse_command_line
// cocolib/cocolib/common/parse_config.cpp:103-158):
//     ulf -config <file> [-key value]... [+flag]...
// Arguments are applied in order ("-config" parses the file at that point; later keys override earlier ones).
// algorithm IBR_color (the default, sr_synthesize_view) or IBR_gradient (IBR_gradient) runs on:
//     lf_name     input views, printf pattern over s = s_min..s_max except s_rmv (PNG or PFM)
//     tau_name    warps tau_%02i.pfm (tau_x, tau_y, deformation)
//     dpart_name  partial_tau_%02i.pfm (sigma_z, dtau_x/dz, dtau_y/dz)
//     init_name   optional starting image (PFM)
//     outdir / outfile   result image (PNG or PFM by extension) and outdir/output.pfm
// Options of this library: -faithful 0|1, -early_exit 0|1, -cg_max_iter n, -cg_gap_tol x, -device n.
#include "lfrv.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

static void die(const char *what) {
    std::fprintf(stderr, "ulf: %s: %s\n", what, lfrv_last_error());
    std::exit(1);
}

static bool ends_with(const std::string &s, const char *suffix) {
    const size_t n = std::strlen(suffix);
    return s.size() >= n && s.compare(s.size() - n, n, suffix) == 0;
}

static std::string key(const char *k) {
    char buf[1024];
    return lfrv_config_get_string(k, buf, sizeof(buf)) == LFRV_OK ? std::string(buf) : std::string();
}

static std::string fmt(const std::string &pattern, int i) {
    char buf[2048];
    std::snprintf(buf, sizeof(buf), pattern.c_str(), i);
    return buf;
}

// Reads one image as 3 x h x w floats (PNG or PFM by extension); sets w, h on the first call.
static void read_image(const std::string &path, int channels, int &w, int &h, std::vector<float> &out) {
    int iw = 0, ih = 0, c = 0;
    if (ends_with(path, ".png") || ends_with(path, ".PNG")) {
        if (lfrv_png_read(path.c_str(), &iw, &ih, nullptr, 0) != LFRV_OK) die(path.c_str());
        c = 3;
    } else {
        if (lfrv_pfm_read(path.c_str(), &iw, &ih, &c, nullptr, 0) != LFRV_OK) die(path.c_str());
    }
    if (w == 0 && h == 0) {
        w = iw;
        h = ih;
    }
    if (iw != w || ih != h) {
        std::fprintf(stderr, "ulf: %s is %d x %d, expected %d x %d\n", path.c_str(), iw, ih, w, h);
        std::exit(1);
    }
    std::vector<float> img((size_t)c * iw * ih);
    const int rc = (c == 3 && (ends_with(path, ".png") || ends_with(path, ".PNG")))
                       ? lfrv_png_read(path.c_str(), &iw, &ih, img.data(), img.size())
                       : lfrv_pfm_read(path.c_str(), &iw, &ih, &c, img.data(), img.size());
    if (rc != LFRV_OK) die(path.c_str());
    const size_t n = (size_t)iw * ih;
    for (int k = 0; k < channels; ++k) {
        const float *src = img.data() + (size_t)(c == 1 ? 0 : k) * n;  // grey PFM replicated (gsl_image_load_pfm)
        out.insert(out.end(), src, src + n);
    }
}

int main(int argc, char **argv) {
    // Sequence of command-line switches as a config file, so "-config" includes keep their position.
    char tmpl[] = "/tmp/ulf_args_XXXXXX";
    const int fd = mkstemp(tmpl);
    if (fd < 0) {
        std::perror("ulf");
        return 1;
    }
    FILE *f = fdopen(fd, "w");
    int device = 0;
    for (int i = 1; i < argc; ++i) {
        if (argv[i][0] == '-' && i + 1 < argc) {
            if (!std::strcmp(argv[i] + 1, "device")) device = std::atoi(argv[i + 1]);
            std::fprintf(f, "%s %s\n", argv[i] + 1, argv[i + 1]);
            ++i;
        } else if (argv[i][0] == '+') {
            std::fprintf(f, "%s 1\n", argv[i] + 1);
        }
    }
    std::fclose(f);
    lfrv_config cfg;
    lfrv_config_default(&cfg);
    const int prc = lfrv_config_parse_file(tmpl, &cfg);
    std::remove(tmpl);
    if (prc != LFRV_OK) die("config");
    int v = 0;
    if (lfrv_config_get_int("faithful", &v) == LFRV_OK) cfg.faithful = v;
    if (lfrv_config_get_int("early_exit", &v) == LFRV_OK) cfg.early_exit = v;
    if (lfrv_config_get_int("cg_max_iter", &v) == LFRV_OK) cfg.cg_max_iter = v;
    if (!key("cg_gap_tol").empty()) cfg.cg_gap_tol = std::atof(key("cg_gap_tol").c_str());
    cfg.nchannels = cfg.nchannels ? cfg.nchannels : 3;
    const std::string algorithm = key("algorithm").empty() ? "IBR_color" : key("algorithm");
    if (algorithm != "IBR_color" && algorithm != "IBR_gradient") {
        std::fprintf(stderr, "ulf: algorithm %s is not part of this path\n", algorithm.c_str());
        return 1;
    }
    int s_min = -1, s_max = -1, s_rmv = -1;
    lfrv_config_get_int("s_min", &s_min);
    lfrv_config_get_int("s_max", &s_max);
    lfrv_config_get_int("s_rmv", &s_rmv);
    if (s_min < 0 || s_max < s_min) {
        std::fprintf(stderr, "ulf: s_min / s_max missing\n");
        return 1;
    }
    int w = cfg.w, h = cfg.h;
    std::vector<float> views, tau, dpart;
    int nv = 0;
    for (int s = s_min; s <= s_max; ++s) {
        if (s == s_rmv) continue;  // the view to synthesise (sources/import.cpp:146)
        read_image(fmt(key("lf_name"), s), 3, w, h, views);
        read_image(fmt(key("tau_name"), s), 3, w, h, tau);
        read_image(fmt(key("dpart_name"), s), 3, w, h, dpart);
        ++nv;
    }
    cfg.w = w;
    cfg.h = h;
    cfg.nviews = nv;
    const int W = w * cfg.dsf, H = h * cfg.dsf;
    std::vector<float> init;
    const std::string init_name = key("init_name");
    if (!init_name.empty()) {
        FILE *t = std::fopen(init_name.c_str(), "rb");
        if (t) {
            std::fclose(t);
            int iw = W, ih = H;
            read_image(init_name, 3, iw, ih, init);
        }
    }
    lfrv_ctx *ctx = nullptr;
    if (lfrv_ctx_create(&ctx, device) != LFRV_OK) die("device");
    std::vector<float> out(3 * (size_t)W * H);
    lfrv_stats st = {};
    const int rc = (algorithm == "IBR_color")
                       ? lfrv_ibr_color(ctx, &cfg, views.data(), tau.data(), 3, dpart.data(),
                                        init.empty() ? nullptr : init.data(), out.data(), &st)
                       : lfrv_ibr_gradient(ctx, &cfg, views.data(), tau.data(), 3, dpart.data(),
                                           init.empty() ? nullptr : init.data(), out.data(), &st);
    if (rc != LFRV_OK) die(algorithm.c_str());
    lfrv_ctx_destroy(ctx);
    std::string outdir = key("outdir");
    if (!outdir.empty() && outdir.back() != '/') outdir += "/";
    if (lfrv_pfm_write((outdir + "output.pfm").c_str(), W, H, 3, out.data()) != LFRV_OK) die("output.pfm");
    const std::string outfile = key("outfile");
    if (!outfile.empty()) {
        const std::string p = outdir + outfile;
        const int wrc = ends_with(p, ".pfm") ? lfrv_pfm_write(p.c_str(), W, H, 3, out.data())
                                             : lfrv_png_write(p.c_str(), W, H, out.data());
        if (wrc != LFRV_OK) die(p.c_str());
    }
    std::printf("%s: %d views %dx%d -> %dx%d, %d iterations, %.3f ms on the device, %d kernels\n",
                algorithm.c_str(), nv, w, h, W, H, st.outer_iterations, st.seconds * 1e3, st.kernel_launches);
    return 0;
}
