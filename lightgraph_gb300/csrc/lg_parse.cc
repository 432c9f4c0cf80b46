// Host helpers that mirror the reference's scene description: Shader defaults
// and setters (src/Shader.h:123-211), SceneSettings defaults
// (src/SceneSettings.h:40-61), the -light and -tempColorRamp parsers
// (src/main.cc:214-319) and the light transforms (src/Light.h:56-126,
// src/main.cc:244-269). The CLI and the Python mirror both call these, so a
// scene string means the same thing on every path.
#include <cmath>
#include <cstring>
#include <sstream>
#include <string>
#include <vector>

#include "lightgraph_c.h"

namespace {

constexpr double kPi = 3.14159265358979323846;

// math::rotation<Mat4d>(axis, angle), 3x3 part, row-vector convention.
void rotation(int axis, double ang, double R[3][3]) {
    const double c = std::cos(ang), s = std::sin(ang);
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[i][j] = (i == j) ? 1.0 : 0.0;
    if (axis == 0) { R[1][1] = c; R[1][2] = s; R[2][1] = -s; R[2][2] = c; }
    else if (axis == 1) { R[0][0] = c; R[0][2] = -s; R[2][0] = s; R[2][2] = c; }
    else { R[0][0] = c; R[0][1] = s; R[1][0] = -s; R[1][1] = c; }
}

void matmul3(const double A[3][3], const double B[3][3], double C[3][3]) {
    double T[3][3];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) T[i][j] = A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j];
    std::memcpy(C, T, sizeof T);
}

// row vector times matrix
void vecmat(const double v[3], const double M[3][3], double out[3]) {
    for (int j = 0; j < 3; ++j) out[j] = v[0] * M[0][j] + v[1] * M[1][j] + v[2] * M[2][j];
}

std::vector<std::string> split(const std::string& s, char sep) {
    std::vector<std::string> out;
    std::stringstream ss(s);
    while (ss.good()) {
        std::string sub;
        std::getline(ss, sub, sep);
        out.push_back(sub);
    }
    return out;
}

// strToVec (src/main.cc:214-229): "a" -> (a,a,a), "a,b,c" -> (a,b,c)
bool str_to_vec(const std::string& s, double out[3]) {
    try {
        std::vector<std::string> p = split(s, ',');
        if (p.size() == 1) {
            out[0] = out[1] = out[2] = std::stod(p[0]);
            return true;
        }
        if (p.size() < 3) return false;
        for (int k = 0; k < 3; ++k) out[k] = std::stod(p[k]);
        return true;
    } catch (...) {
        return false;
    }
}

}  // namespace

extern "C" void lg_shader_default(lg_shader* s) {
    if (!s) return;
    std::memset(s, 0, sizeof *s);
    s->density_scale = 1.0;
    s->density_max = 100.0;
    s->shadow_density_scale = 1.0;
    s->scatter_density_scale = 0.35;
    s->scatter_density_min = 0.025;
    const double absorption[3] = {0.1, 0.1, 0.1}, scattering[3] = {1.5, 1.5, 1.5}, color[3] = {1, 1, 1};
    lg_shader_set_coefficients(s, absorption, scattering, color);
    s->emission_scale = 0.0;
    s->scatter_scale = 4.0;
    s->scatter_density_mask_power = 0.25;
    s->ramp_n = 0;
    s->ramp_in = 0.0;
    s->ramp_out = 1.0;
}

extern "C" void lg_shader_set_coefficients(lg_shader* s, const double absorption[3], const double scattering[3],
                                           const double volume_color[3]) {
    if (!s) return;
    for (int c = 0; c < 3; ++c) {
        s->scattering[c] = scattering[c];
        s->albedo[c] = (volume_color[c] * scattering[c]) / (scattering[c] + absorption[c]);
        s->extinction[c] = -(scattering[c] + absorption[c]);
    }
}

extern "C" void lg_settings_default(lg_settings* o) {
    if (!o) return;
    std::memset(o, 0, sizeof *o);
    o->cutoff = 0.005;
    o->step[0] = 1.0;
    o->step[1] = 3.0;
    o->iter = 10;
    o->scatter_grid_res_factor = 4;
    o->pts_per_kernel = 3;
    o->seed = 0;
}

extern "C" void lg_camera_default(lg_camera* c) {
    if (!c) return;
    std::memset(c, 0, sizeof *c);
    c->focal = 50.0;
    c->aperture = 36.0;
    c->znear = 1.0e-3;
    c->zfar = 3.4028234663852886e38;  // std::numeric_limits<float>::max()
    c->width = 960;
    c->height = 540;
    c->samples = 1;
}

extern "C" lg_status lg_parse_light(const char* spec, lg_light* out) {
    if (!spec || !out) return LG_ERR_INVALID;
    std::memset(out, 0, sizeof *out);
    const std::vector<std::string> p = split(spec, ':');
    try {
        if (p.size() < 5) return LG_ERR_INVALID;
        const double yrot = std::stod(p[1]) / 180.0 * kPi;
        double color[3];
        if (!str_to_vec(p[2], color)) return LG_ERR_INVALID;
        const double intensity = (double)(float)std::stod(p[3]);  // Light::mIntensity is a float
        double Ry[3][3];
        rotation(1, yrot, Ry);  // yRotXform
        for (int c = 0; c < 3; ++c) out->color[c] = color[c];
        out->intensity = intensity;
        out->samples = 1;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) out->rot[i * 3 + j] = Ry[i][j];
        if (p[0] == "env") {
            // env:yRot:color:intensity:samples:exrFile (src/main.cc:244-254)
            out->type = LG_LIGHT_ENV;
            out->samples = std::stoi(p[4]);
            if (out->samples < 1) return LG_ERR_INVALID;
            return LG_OK;
        }
        if (p[0] == "dir") {
            // dir:yRot:color:intensity:rx,ry,rz (src/main.cc:255-269)
            double rot[3];
            if (!str_to_vec(p[4], rot)) return LG_ERR_INVALID;
            double M[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
            for (int a = 0; a < 3; ++a) {
                double R[3][3];
                rotation(a, -rot[a] * kPi / 180.0, R);  // AffineMap::accumPostRotation
                matmul3(M, R, M);
            }
            matmul3(M, Ry, M);  // orientXform.getMat4() * yRotXform(yRot)
            const double d0[3] = {0.0, 0.0, -1.0};
            double d[3];
            vecmat(d0, M, d);
            const double len = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            for (int c = 0; c < 3; ++c) out->dir[c] = d[c] / len;
            out->type = LG_LIGHT_DISTANT;
            return LG_OK;
        }
        if (p[0] == "point") {
            // point:yRot:color:intensity:x,y,z -- PointLight (src/Light.h:56-91)
            // has no command-line syntax in the reference; this one follows dir's
            double pos[3];
            if (!str_to_vec(p[4], pos)) return LG_ERR_INVALID;
            vecmat(pos, Ry, out->pos);
            out->type = LG_LIGHT_POINT;
            return LG_OK;
        }
    } catch (...) {
        return LG_ERR_INVALID;
    }
    return LG_ERR_INVALID;
}

extern "C" lg_status lg_parse_color_ramp(const char* spec, lg_shader* s) {
    // posTicks/colorTicks/minTempRemap/maxTempRemap (src/main.cc:280-319)
    if (!spec || !s) return LG_ERR_INVALID;
    const std::vector<std::string> parts = split(spec, '/');
    if (parts.size() != 4) return LG_ERR_INVALID;
    try {
        const std::vector<std::string> pos = split(parts[0], ',');
        const std::vector<std::string> col = split(parts[1], ':');
        if (pos.size() != col.size() || pos.size() > LG_MAX_RAMP_KEYS) return LG_ERR_INVALID;
        for (size_t k = 0; k < pos.size(); ++k) {
            s->ramp_pos[k] = std::stod(pos[k]);
            if (!str_to_vec(col[k], s->ramp_color[k])) return LG_ERR_INVALID;
        }
        s->ramp_n = (int32_t)pos.size();
        s->ramp_in = std::stod(parts[2]);
        s->ramp_out = std::stod(parts[3]);
    } catch (...) {
        return LG_ERR_INVALID;
    }
    return LG_OK;
}
