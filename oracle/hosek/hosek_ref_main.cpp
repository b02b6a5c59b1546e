// hosek_ref_main.cpp — pins the Hosek-Wilkie coefficient evaluation against
// the reference's own C++ and writes the derived coefficient table
// (TEST INFRASTRUCTURE; built only where the reference tree is present, by
// oracle/hosek/build_ref.sh, into oracle/_ref/).
//
// It compiles the reference's evaluate_spline/evaluate
// (src/engine/gfx/hosek_wilkie_sky_model.cpp:41-67, extracted verbatim into
// oracle/_ref/ by the build script, never committed) together with the
// reference's data table include/gfx/hosek_data_rgb.inl (Hosek & Wilkie 2012,
// third-party data, included from where it lies), and checks the oracle's
// restatement (restated_evaluate below) bit for bit against it.
//
// Outputs (committed; derived data only, no table rows):
//   helios_gb300/csrc/hosek_table.inc — each raw coefficient's spline A..I,Z
//       (RGB) sampled at six points of elevation^(1/3), for ground albedo 0
//       and 1 and turbidity 1..10 (the quintic is exact from six samples);
//   tests/golden/hosek_coeffs.json — the reference's normalised coefficients
//       (evaluate + the luminance normalisation of HosekWilkieSkyModel::update)
//       at on- and off-grid sun elevations, fractional turbidities and
//       several ground albedos.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>

namespace glm {
template <typename T> T clamp(T x, T lo, T hi) { return std::min(std::max(x, lo), hi); }
}
#define _USE_MATH_DEFINES
#include "hosek_data_rgb.inl"
#include "hw_eval_ref.inc"  // reference evaluate_spline + evaluate (extracted)

// Restatement (the oracle's): a quintic Bernstein spline in elevation^(1/3),
// bilinear in (albedo, turbidity).
static double restated_spline(const double* s, size_t stride, double x) {
    return 1 * pow(1 - x, 5) * s[0 * stride] + 5 * pow(1 - x, 4) * pow(x, 1) * s[1 * stride] +
           10 * pow(1 - x, 3) * pow(x, 2) * s[2 * stride] + 10 * pow(1 - x, 2) * pow(x, 3) * s[3 * stride] +
           5 * pow(1 - x, 1) * pow(x, 4) * s[4 * stride] + 1 * pow(x, 5) * s[5 * stride];
}
static double restated_evaluate(const double* d, size_t stride, float turbidity, float albedo, float sun_theta) {
    double ek = pow(std::max<float>(0.f, 1.f - sun_theta / (M_PI / 2.f)), 1.f / 3.0f);
    int t0 = std::min(std::max(static_cast<int>(turbidity), 1), 10);
    int t1 = std::min(t0 + 1, 10);
    float tk = std::min(std::max(turbidity - t0, 0.f), 1.f);
    const double* a0 = d;
    const double* a1 = d + stride * 6 * 10;
    double a0t0 = restated_spline(a0 + stride * 6 * (t0 - 1), stride, ek);
    double a1t0 = restated_spline(a1 + stride * 6 * (t0 - 1), stride, ek);
    double a0t1 = restated_spline(a0 + stride * 6 * (t1 - 1), stride, ek);
    double a1t1 = restated_spline(a1 + stride * 6 * (t1 - 1), stride, ek);
    return a0t0 * (1 - albedo) * (1 - tk) + a1t0 * albedo * (1 - tk) + a0t1 * (1 - albedo) * tk + a1t1 * albedo * tk;
}

// Raw coefficients in UBO order A..I, Z (H and I swapped in the dataset,
// hosek_wilkie_sky_model.cpp:672-676); ref selects the reference function.
static void coeffs(bool ref, float turbidity, float albedo, float theta, float out[30]) {
    static const int src[9] = {0, 1, 2, 3, 4, 5, 6, 8, 7};
    for (int p = 0; p < 9; ++p)
        for (int c = 0; c < 3; ++c)
            out[p * 3 + c] = (float)(ref ? evaluate(datasetsRGB[c] + src[p], 9, turbidity, albedo, theta)
                                         : restated_evaluate(datasetsRGB[c] + src[p], 9, turbidity, albedo, theta));
    for (int c = 0; c < 3; ++c)
        out[27 + c] = (float)(ref ? evaluate(datasetsRGBRad[c], 1, turbidity, albedo, theta)
                                  : restated_evaluate(datasetsRGBRad[c], 1, turbidity, albedo, theta));
}

// hosek_wilkie (hosek_wilkie_sky_model.cpp:71-75), float, per channel.
static float hw(float cos_theta, float gamma, float cos_gamma, const float* k, int c) {
    float A = k[0 + c], B = k[3 + c], C = k[6 + c], D = k[9 + c], E = k[12 + c], F = k[15 + c], G = k[18 + c], H = k[21 + c], I = k[24 + c];
    float chi = (1.f + cos_gamma * cos_gamma) / powf(1.f + H * H - 2.f * cos_gamma * H, 1.5f);
    return (1.f + A * expf(B / (cos_theta + 0.01f))) * (C + D * expf(E * gamma) + F * (cos_gamma * cos_gamma) + G * chi + I * sqrtf(std::max(0.f, cos_theta)));
}

// The spline of one (coefficient, albedo a in {0, 1}, turbidity t in 1..10)
// sampled at e_j = j / 5, j = 0..5 (e = elevation^(1/3)): six values fix the
// quintic exactly, so the library evaluates any sun angle from them.
static double node_value(const double* dataset, size_t stride, int a, int t, int j) {
    const double* base = dataset + stride * 6 * 10 * a + stride * 6 * (t - 1);
    return evaluate_spline(base, stride, j / 5.0);
}

int main(int argc, char** argv) {
    if (argc < 3) { fprintf(stderr, "usage: %s table.inc golden.json\n", argv[0]); return 2; }
    static const int src[9] = {0, 1, 2, 3, 4, 5, 6, 8, 7};
    FILE* ft = fopen(argv[1], "w");
    fprintf(ft, "// Generated by oracle/hosek/hosek_ref_main.cpp from the Hosek-Wilkie RGB model\n"
                "// (Hosek & Wilkie 2012): the quintic spline of each raw coefficient A..I,Z (RGB,\n"
                "// UBO order) sampled at elevation^(1/3) = j / 5, j = 0..5, for ground albedo\n"
                "// {0, 1} and turbidity 1..10. Derived data (samples, not the model's table).\n"
                "static const double kHosekNodes[2][10][6][30] = {\n");
    for (int a = 0; a < 2; ++a) {
        fprintf(ft, "{\n");
        for (int t = 1; t <= 10; ++t) {
            fprintf(ft, " {\n");
            for (int j = 0; j <= 5; ++j) {
                fprintf(ft, "  {");
                for (int q = 0; q < 30; ++q) {
                    double v = q < 27 ? node_value(datasetsRGB[q % 3] + src[q / 3], 9, a, t, j)
                                      : node_value(datasetsRGBRad[q - 27], 1, a, t, j);
                    fprintf(ft, "%.17g%s", v, q < 29 ? "," : "");
                }
                fprintf(ft, "}%s\n", j < 5 ? "," : "");
            }
            fprintf(ft, " }%s\n", t < 10 ? "," : "");
        }
        fprintf(ft, "}%s\n", a < 1 ? "," : "");
    }
    fprintf(ft, "};\n");
    fclose(ft);
    // golden: the reference's evaluate + update normalisation at on- and
    // off-grid sun elevations, integer and fractional turbidities, several
    // ground albedos; also pins the restatement bit for bit on each case
    long mismatches = 0, cases = 0;
    FILE* fg = fopen(argv[2], "w");
    fprintf(fg, "{\"source\": \"reference evaluate (hosek_wilkie_sky_model.cpp:41-67) + update normalisation (:658-686)\",\n \"normalized_sun_y\": 1.15, \"cases\": [\n");
    const float elevs[9] = {0.5f, 10.f, 12.3f, 30.f, 37.77f, 45.f, 61.9f, 80.f, 89.5f};
    const float turbs[7] = {1.f, 2.5f, 3.f, 4.f, 4.7f, 7.25f, 10.f};
    const float albs[4] = {0.f, 0.1f, 0.35f, 1.f};
    bool first = true;
    for (float tb : turbs)
        for (float al : albs)
            for (float el : elevs) {
                if (al != 0.1f && (el == 10.f || el == 45.f || el == 80.f)) continue;
                float e = el * (float)M_PI / 180.f;
                float dir[3] = {cosf(e) * 0.6f, sinf(e), cosf(e) * 0.8f};
                float theta = std::acos(std::min(std::max(dir[1], 0.f), 1.f));
                float k[30], r[30];
                coeffs(true, tb, al, theta, k);
                coeffs(false, tb, al, theta, r);
                if (memcmp(k, r, sizeof(k)) != 0) ++mismatches;
                ++cases;
                float S[3];
                for (int c = 0; c < 3; ++c) S[c] = hw(std::cos(theta), 0, 1.f, k, c) * k[27 + c];
                float lum = S[0] * 0.2126f + S[1] * 0.7152f + S[2] * 0.0722f;
                for (int c = 0; c < 3; ++c) { k[27 + c] /= lum; k[27 + c] *= 1.15f; }
                fprintf(fg, "%s  {\"turbidity\": %.9g, \"albedo\": %.9g, \"elevation_deg\": %.9g, \"sun_direction\": [%.9g, %.9g, %.9g], \"coeffs\": [",
                        first ? "" : ",\n", tb, al, el, dir[0], dir[1], dir[2]);
                for (int q = 0; q < 30; ++q) fprintf(fg, "%.9g%s", k[q], q < 29 ? ", " : "");
                fprintf(fg, "]}");
                first = false;
            }
    fprintf(fg, "\n]}\n");
    fclose(fg);
    printf("restated vs reference evaluate mismatches: %ld of %ld cases\n", mismatches, cases);
    return mismatches == 0 ? 0 : 1;
}
