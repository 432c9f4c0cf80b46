// lightgraph: command-line renderer with the reference's flags (src/main.cc:138-470)
// and its three stages (LightGraph solve, scatter-grid splat, render), running on
// the GPU through the C ABI.
//
// OpenVDB is not available, so the volume comes from -synthetic
// {sphere,cumulus}:<res> (seeded fBm, see lightgraph_scene.h) or from -rawIn
// <file>:<res>:<voxelSize> (a dense res^3 float32 array, x fastest). Points are
// thrown by the reference's dart throwing on the GPU (default), or injected:
// -points <file> (float32 x,y,z triples) or uniform interior samples
// (-numPoints, -seed). Output is an uncompressed multi-layer EXR with the
// reference's 13 channels (src/Image.h:47-62).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <string>
#include <vector>

#include "lightgraph_c.h"
#include "lightgraph_scene.h"

namespace {

void print_help() {
    std::cout <<
        "-vdbIn                  : not supported (no OpenVDB in this binary); use -synthetic or -rawIn\n"
        "-synthetic              : kind:res, kind in {sphere, cumulus}   ex: cumulus:512\n"
        "-rawIn                  : file:res:voxelSize (dense float32 res^3, x fastest)\n"
        "-exrOut                 : output EXR (13 channels, uncompressed)\n"
        "-camPos -camRot         : float,float,float\n"
        "-camYRot                : float\n"
        "-resWidth -resHeight    : int\n"
        "-focal                  : float (mm)\n"
        "-samples                : antialiasing samples per pixel\n"
        "-primaryStep -shadowStep: voxels per sample\n"
        "-cutoff                 : float\n"
        "-light                  : dir:yRot:r,g,b:intensity:rx,ry,rz | point:yRot:r,g,b:intensity:x,y,z |\n"
        "                          env:yRot:r,g,b:intensity:samples:sky (synthetic sky map) or a path\n"
        "                          to an uncompressed EXR env map\n"
        "-iter                   : number of LightGraphs\n"
        "-numPoints              : uniform interior points per LightGraph instead of dart throwing\n"
        "-connectRadius          : connection radius in world units for -numPoints/-points\n"
        "                          (default 1.7 x spacing)\n"
        "-points                 : float32 x,y,z file (one graph per -iter slice)\n"
        "                          (default: the reference's dart throwing, on the GPU)\n"
        "-geoDump                : write the LightGraph geometry to geoDump/ as ASCII files\n"
        "-seed                   : seed of the points and of the render random streams\n"
        "-scatterGridResFactor -ptsPerKernel -densityScale -densityMax -shadowDensityScale\n"
        "-scatterDensityScale -scatterDensityMin -absorption -scattering -volumeColor\n"
        "-emissionScale -scatterScale -scatterDensityMaskPower -tempColorRamp\n"
        "-precision              : fp32 | fp16 | bf16 grid storage\n"
        "-v -h -help --help\n";
}

bool vec3(const char* s, double out[3]) {
    double a, b, c;
    if (std::sscanf(s, "%lf,%lf,%lf", &a, &b, &c) == 3) { out[0] = a; out[1] = b; out[2] = c; return true; }
    if (std::sscanf(s, "%lf", &a) == 1) { out[0] = out[1] = out[2] = a; return true; }
    return false;
}

// Minimal OpenEXR writer: scanline, NO_COMPRESSION, FLOAT channels in
// alphabetical order, one line per block.
double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

}  // namespace

// Edge of the cube that holds one point on average over the points' bbox
// (0.1 for fewer than two points or a flat box).
static double mean_spacing(int64_t n, const float* p) {
    if (n < 2) return 0.1;
    double lo[3] = {p[0], p[1], p[2]}, hi[3] = {p[0], p[1], p[2]};
    for (int64_t i = 1; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            lo[a] = std::min(lo[a], (double)p[3 * i + a]);
            hi[a] = std::max(hi[a], (double)p[3 * i + a]);
        }
    const double vol = (hi[0] - lo[0]) * (hi[1] - lo[1]) * (hi[2] - lo[2]);
    return vol > 0 ? std::cbrt(vol / (double)n) : 0.1;
}

int main(int argc, char** argv) {
    lg_shader shader;
    lg_shader_default(&shader);
    lg_settings opts;
    lg_settings_default(&opts);
    lg_camera cam;
    lg_camera_default(&cam);
    std::vector<lg_light> lights;
    std::string exr_out = "lightgraph.exr", synthetic = "sphere:128", raw_in, points_file;
    double absorption[3] = {0.1, 0.1, 0.1}, scattering[3] = {1.5, 1.5, 1.5}, color[3] = {1, 1, 1};
    int num_points = 0, dtype = LG_DTYPE_F32;
    bool geo_dump = false;
    double connect_radius = -1.0;
    bool verbose = false, need_env = false;
    std::string env_file;
    for (int i = 1; i < argc; ++i) {
        const std::string a = argv[i];
        auto next = [&]() -> const char* {
            if (i + 1 >= argc) { std::cerr << a << " needs a value\n"; std::exit(1); }
            return argv[++i];
        };
        double v3[3];
        if (a == "-h" || a == "-help" || a == "--help") { print_help(); return 0; }
        else if (a == "-v") verbose = true;
        else if (a == "-geoDump") geo_dump = true;
        else if (a == "-vdbIn") { std::cerr << "-vdbIn needs OpenVDB, which this binary does not link; use -synthetic or -rawIn\n"; return 1; }
        else if (a == "-synthetic") synthetic = next();
        else if (a == "-rawIn") raw_in = next();
        else if (a == "-exrOut") exr_out = next();
        else if (a == "-camPos") { if (!vec3(next(), v3)) return 1; std::memcpy(cam.translate, v3, sizeof v3); }
        else if (a == "-camRot") { if (!vec3(next(), v3)) return 1; std::memcpy(cam.rotate, v3, sizeof v3); }
        else if (a == "-camYRot") cam.y_rotate = std::atof(next());
        else if (a == "-resWidth") cam.width = std::atoi(next());
        else if (a == "-resHeight") cam.height = std::atoi(next());
        else if (a == "-focal") cam.focal = (float)std::atof(next());
        else if (a == "-samples") cam.samples = std::max(0, std::atoi(next()));
        else if (a == "-primaryStep") opts.step[0] = std::atof(next());
        else if (a == "-shadowStep") opts.step[1] = std::atof(next());
        else if (a == "-cutoff") opts.cutoff = std::atof(next());
        else if (a == "-light") {
            lg_light L;
            const char* spec = next();
            if (lg_parse_light(spec, &L) != LG_OK) { std::cout << spec << " is not a valid light!\n"; continue; }
            if (L.type == LG_LIGHT_ENV) {
                need_env = true;
                // env:yRot:color:intensity:samples:file -- "sky" is the synthetic map
                const std::string sp(spec);
                const std::string file = sp.substr(sp.find_last_of(':') + 1);
                if (file != "sky") env_file = file;
            }
            lights.push_back(L);
        }
        else if (a == "-iter") opts.iter = std::atoi(next());
        else if (a == "-scatterGridResFactor") opts.scatter_grid_res_factor = std::atoi(next());
        else if (a == "-ptsPerKernel") opts.pts_per_kernel = std::atoi(next());
        else if (a == "-densityScale") shader.density_scale = std::stod(next());
        else if (a == "-densityMax") shader.density_max = std::stod(next());
        else if (a == "-shadowDensityScale") shader.shadow_density_scale = std::stod(next());
        else if (a == "-scatterDensityScale") shader.scatter_density_scale = std::stod(next());
        else if (a == "-scatterDensityMin") shader.scatter_density_min = std::stod(next());
        else if (a == "-absorption") { if (!vec3(next(), absorption)) return 1; }
        else if (a == "-scattering") { if (!vec3(next(), scattering)) return 1; }
        else if (a == "-volumeColor") { if (!vec3(next(), color)) return 1; }
        else if (a == "-emissionScale") shader.emission_scale = std::stod(next());
        else if (a == "-scatterScale") shader.scatter_scale = std::stod(next());
        else if (a == "-scatterDensityMaskPower") shader.scatter_density_mask_power = std::stod(next());
        else if (a == "-tempColorRamp") { if (lg_parse_color_ramp(next(), &shader) != LG_OK) { std::cerr << "bad ramp\n"; return 1; } }
        else if (a == "-numPoints") num_points = std::atoi(next());
        else if (a == "-connectRadius") connect_radius = std::atof(next());
        else if (a == "-points") points_file = next();
        else if (a == "-seed") opts.seed = (uint64_t)std::strtoull(next(), nullptr, 10);
        else if (a == "-precision") {
            const std::string p = next();
            dtype = p == "fp16" ? LG_DTYPE_F16 : (p == "bf16" ? LG_DTYPE_BF16 : LG_DTYPE_F32);
        }
        else { std::cout << a << " is not a valid option\n"; return 1; }
    }
    lg_shader_set_coefficients(&shader, absorption, scattering, color);

    // volume
    int res = 128;
    double voxel = 0.01;
    std::vector<float> dens;
    if (!raw_in.empty()) {
        char file[4096];
        if (std::sscanf(raw_in.c_str(), "%4095[^:]:%d:%lf", file, &res, &voxel) != 3) { std::cerr << "bad -rawIn\n"; return 1; }
        dens.resize((size_t)res * res * res);
        std::ifstream f(file, std::ios::binary);
        if (!f.read((char*)dens.data(), dens.size() * 4)) { std::cerr << "cannot read " << file << "\n"; return 1; }
    } else {
        char kind[64];
        if (std::sscanf(synthetic.c_str(), "%63[^:]:%d", kind, &res) != 2) { std::cerr << "bad -synthetic\n"; return 1; }
        voxel = 1.28 / res;
        dens.resize((size_t)res * res * res);
        const bool cumulus = std::string(kind) == "cumulus";
        lgs_volume(cumulus ? LGS_VOLUME_CUMULUS : LGS_VOLUME_SPHERE_FBM, res, cumulus ? 6 : 4, cumulus ? 1 : 0, 1.0,
                   nullptr, dens.data());
    }
    lg_ctx* ctx = nullptr;
    if (lg_create(0, &ctx) != LG_OK) { std::cerr << "no CUDA device\n"; return 1; }
    auto check = [&](lg_status s, const char* what) {
        if (s != LG_OK) { std::cerr << what << ": " << lg_last_error(ctx) << "\n"; std::exit(1); }
    };
    lg_grid_desc gd;
    std::memset(&gd, 0, sizeof gd);
    for (int a = 0; a < 3; ++a) { gd.dims[a] = res; gd.origin[a] = -res / 2; }
    gd.voxel_size = voxel;
    check(lg_upload_grid(ctx, LG_GRID_DENSITY, &gd, dens.data(), dtype), "density upload");
    std::vector<float> env;
    int ew = 512, eh = 256;
    if (need_env && !env_file.empty()) {
        // an uncompressed EXR env map, read as readExr does (half RGBA)
        int32_t w = 0, h = 0;
        if (lg_read_exr_rgba(env_file.c_str(), &w, &h, nullptr) != LG_OK) {
            std::cerr << "cannot read the env map " << env_file << " (uncompressed scanline EXR only)\n";
            return 1;
        }
        std::vector<float> rgba((size_t)w * h * 4);
        lg_read_exr_rgba(env_file.c_str(), &w, &h, rgba.data());
        ew = w;
        eh = h;
        env.resize((size_t)w * h * 3);
        for (size_t p = 0; p < (size_t)w * h; ++p)
            for (int c = 0; c < 3; ++c) env[3 * p + c] = rgba[4 * p + c];
    } else if (need_env) {
        env.resize((size_t)ew * eh * 3);
        lgs_envmap(ew, eh, 30.0, 60.0, 2.0, 50.0, env.data());
    }
    check(lg_set_lights(ctx, lights.data(), (int)lights.size(), need_env ? env.data() : nullptr, ew, eh), "lights");
    check(lg_set_shader(ctx, &shader), "shader");
    check(lg_set_settings(ctx, &opts), "settings");

    // points: one graph per iteration
    std::vector<float> pts;
    std::vector<int64_t> offs(1, 0);
    const bool dart = points_file.empty() && num_points <= 0;
    if (dart) {
        // LightGraph::scatterPoints for every iteration, then buildGraph
        lg_scatter_opts so;
        lg_scatter_opts_default(&so);
        std::vector<int32_t> counts(opts.iter);
        const double t0 = now_s();
        check(lg_scatter_graphs(ctx, &so, 0, opts.iter, 12, counts.data()), "dart throwing");
        for (int g = 0; g < opts.iter; ++g) offs.push_back(offs.back() + counts[g]);
        if (verbose) std::cout << "Point Cloud Creation: " << (now_s() - t0) << " sec" << std::endl;
    } else if (!points_file.empty()) {
        std::ifstream f(points_file, std::ios::binary | std::ios::ate);
        const size_t n = (size_t)f.tellg() / 12;
        f.seekg(0);
        pts.resize(n * 3);
        f.read((char*)pts.data(), n * 12);
        for (int g = 0; g < opts.iter; ++g) offs.push_back((int64_t)(n * (g + 1) / opts.iter));
    } else {
        for (int g = 0; g < opts.iter; ++g) {
            std::vector<float> p((size_t)num_points * 3);
            const int64_t got = lgs_points(dens.data(), res, voxel, num_points, opts.seed * 1000003ull + g, 0.001,
                                           (int64_t)num_points * 10000, p.data());
            pts.insert(pts.end(), p.begin(), p.begin() + 3 * got);
            offs.push_back(offs.back() + got);
        }
    }
    std::vector<float> r2(dart ? 0 : opts.iter);
    for (int g = 0; g < (dart ? 0 : opts.iter); ++g) {
        double r = connect_radius;
        if (r <= 0) {
            // 1.7 x the mean spacing of the graph's points (CONNECT_SEARCH_RADIUS_MULT)
            r = 1.7 * mean_spacing(offs[g + 1] - offs[g], pts.data() + 3 * offs[g]);
        }
        r2[g] = (float)r * (float)r;
    }
    const double t0 = now_s();
    if (!dart)
        check(lg_build_graphs(ctx, opts.iter, pts.data(), offs.data(), r2.data(), 12, nullptr, nullptr),
              "build graphs");
    check(lg_solve_graphs(ctx, nullptr), "solve graphs");
    if (geo_dump) {
        // file stem of the volume (the reference uses the .vdb file's stem)
        std::string stem = raw_in.empty() ? synthetic : raw_in.substr(0, raw_in.find(':'));
        stem = stem.substr(stem.find_last_of('/') + 1);
        stem = stem.substr(0, stem.find('.'));
        for (char& c : stem)
            if (c == ':') c = '_';
        check(lg_geo_dump(ctx, "geoDump", stem.c_str(), 0), "geo dump");
    }
    const double t1 = now_s();
    std::cout << "LightGraphs Calculation: " << (t1 - t0) << " sec" << std::endl;
    if (verbose) std::cout << "Point Cloud size: " << offs.back() << std::endl;
    check(lg_splat(ctx, 0.0), "splat");
    const double t2 = now_s();
    std::cout << "Rasterize LightGraphs to Grid: " << (t2 - t1) << " sec" << std::endl;
    const size_t np = (size_t)cam.width * cam.height;
    std::vector<float> rgba(np * 4), direct(np * 4), scatter(np * 4), emission(np * 4);
    check(lg_render(ctx, &cam, rgba.data(), direct.data(), scatter.data(), emission.data()), "render");
    const double t3 = now_s();
    std::cout << "Render: " << (t3 - t2) << " sec" << std::endl;
    // planar channels for the EXR
    std::vector<std::vector<float>> planes(13, std::vector<float>(np));
    for (size_t p = 0; p < np; ++p) {
        for (int c = 0; c < 4; ++c) planes[c][p] = rgba[4 * p + c];
        for (int c = 0; c < 3; ++c) {
            planes[4 + c][p] = direct[4 * p + c];
            planes[7 + c][p] = scatter[4 * p + c];
            planes[10 + c][p] = emission[4 * p + c];
        }
    }
    const char* names[13] = {"R", "G", "B", "A", "direct.R", "direct.G", "direct.B", "scatter.R", "scatter.G",
                             "scatter.B", "emission.R", "emission.G", "emission.B"};
    const float* plane_ptrs[13];
    for (int k = 0; k < 13; ++k) plane_ptrs[k] = planes[k].data();
    if (lg_write_exr(exr_out.c_str(), cam.width, cam.height, 13, names, plane_ptrs) != LG_OK) {
        std::cerr << "cannot write " << exr_out << "\n";
        return 1;
    }
    std::cout << "Writting to Disk: " << exr_out << "\n\n";
    lg_destroy(ctx);
    return 0;
}
