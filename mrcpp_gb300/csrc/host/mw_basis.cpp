// Scaling bases, quadrature, filter tables and the 1D filter primitive.
//
// Follows src/core/LegendreBasis.cpp:60-66, src/core/InterpolatingBasis.cpp:65-86
// and :105-111 (cv maps), src/core/GaussQuadrature.cpp:150-180 (Newton on P_n),
// src/core/MWFilter.cpp:100-133 (sub-filter selection) and :225-244 (H1/G1
// from symmetry), src/utils/math_utils.cpp:175-194 (apply_filter).
#include "mw_host.h"

#include <dlfcn.h>

#include <cstdio>
#include <map>
#include <mutex>

namespace mwh {

namespace {
std::mutex g_mu;
std::string g_table_path;
std::map<std::array<int, 3>, Mat> *g_tables = nullptr;
std::map<std::array<int, 2>, ScalingBasis *> g_bases;

std::string default_table_path() {
    if (const char *e = std::getenv("MWGPU_TABLES")) return e;
    Dl_info info;
    if (dladdr((void *)&default_table_path, &info) && info.dli_fname) {
        std::string so(info.dli_fname);
        auto pos = so.find_last_of('/');
        std::string dir = pos == std::string::npos ? "." : so.substr(0, pos);
        for (const char *rel : {"/data/mwtables.bin", "/../data/mwtables.bin"}) {
            std::string p = dir + rel;
            if (FILE *f = std::fopen(p.c_str(), "rb")) { std::fclose(f); return p; }
        }
    }
    return "mwtables.bin";
}

void load_tables_locked() {
    if (g_tables) return;
    std::string path = g_table_path.empty() ? default_table_path() : g_table_path;
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) throw Error(2, "cannot open MW table file " + path);
    char magic[4];
    int32_t hdr[2];
    if (std::fread(magic, 1, 4, f) != 4 || std::memcmp(magic, "MWTB", 4) != 0 || std::fread(hdr, 4, 2, f) != 2) {
        std::fclose(f);
        throw Error(2, "bad MW table file " + path);
    }
    auto *tabs = new std::map<std::array<int, 3>, Mat>();
    for (int e = 0; e < hdr[1]; e++) {
        int32_t h[5];
        if (std::fread(h, 4, 5, f) != 5) { std::fclose(f); delete tabs; throw Error(2, "truncated MW table file"); }
        int r = h[3], c = h[4];
        std::vector<double> buf((size_t)r * c);
        if (std::fread(buf.data(), 8, buf.size(), f) != buf.size()) { std::fclose(f); delete tabs; throw Error(2, "truncated MW table file"); }
        Mat m(r, c);
        for (int i = 0; i < r; i++)
            for (int j = 0; j < c; j++) m(i, j) = buf[(size_t)i * c + j];
        (*tabs)[{h[0], h[1], h[2]}] = std::move(m);
    }
    std::fclose(f);
    g_tables = tabs;
}

Mat inverse(const Mat &A) {
    int n = A.rows;
    Mat a = A, inv(n, n);
    for (int i = 0; i < n; i++) inv(i, i) = 1.0;
    for (int c = 0; c < n; c++) {
        int p = c;
        for (int r = c + 1; r < n; r++)
            if (std::fabs(a(r, c)) > std::fabs(a(p, c))) p = r;
        if (p != c)
            for (int j = 0; j < n; j++) { std::swap(a(p, j), a(c, j)); std::swap(inv(p, j), inv(c, j)); }
        double d = a(c, c);
        for (int j = 0; j < n; j++) { a(c, j) /= d; inv(c, j) /= d; }
        for (int r = 0; r < n; r++) {
            if (r == c) continue;
            double m = a(r, c);
            if (m == 0.0) continue;
            for (int j = 0; j < n; j++) { a(r, j) -= m * a(c, j); inv(r, j) -= m * inv(c, j); }
        }
    }
    return inv;
}

}  // namespace

double legendre_scaled(int j, double x) {  // sqrt(2j+1) P_j(2x-1)
    double t = 2.0 * x - 1.0, p0 = 1.0, p1 = t;
    if (j == 0) return 1.0;
    for (int m = 2; m <= j; m++) {
        double p2 = ((2.0 * m - 1.0) * t * p1 - (m - 1.0) * p0) / m;
        p0 = p1;
        p1 = p2;
    }
    return std::sqrt(2.0 * j + 1.0) * p1;
}

void set_table_path(const std::string &path) {
    std::lock_guard<std::mutex> lk(g_mu);
    g_table_path = path;
}

const Mat &table(int kind, int type, int k) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_tables_locked();
    auto it = g_tables->find({kind, type, k});
    if (it == g_tables->end())
        throw Error(2, "MW table missing: kind " + std::to_string(kind) + " type " + std::to_string(type) + " order " + std::to_string(k));
    return it->second;
}

void gauss_legendre01(int n, std::vector<double> &x, std::vector<double> &w) {
    x.assign(n, 0.0);
    w.assign(n, 0.0);
    int half = (n + 1) / 2;
    for (int i = 0; i < half; i++) {
        double z = std::cos(pi * (i + 0.75) / (n + 0.5)), dp = 1.0;
        for (int it = 0; it < 100; it++) {
            double p0 = 1.0, p1 = z;
            for (int m = 2; m <= n; m++) {
                double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
                p0 = p1;
                p1 = p2;
            }
            double pn = n == 0 ? 1.0 : p1, pm = n == 0 ? 0.0 : p0;
            if (n == 1) { pn = z; pm = 1.0; }
            dp = n * (z * pn - pm) / (z * z - 1.0);
            double z1 = z;
            z = z1 - pn / dp;
            if (std::fabs(z - z1) <= 1.0e-15) break;
        }
        double p0 = 1.0, p1 = z;
        for (int m = 2; m <= n; m++) {
            double p2 = ((2.0 * m - 1.0) * z * p1 - (m - 1.0) * p0) / m;
            p0 = p1;
            p1 = p2;
        }
        if (n == 1) { p1 = z; p0 = 1.0; }
        dp = n * (z * p1 - p0) / (z * z - 1.0);
        double wt = 1.0 / ((1.0 - z * z) * dp * dp);  // on [0,1]: 2/((1-z^2)dp^2) * 1/2
        x[i] = 0.5 - 0.5 * z;
        x[n - 1 - i] = 0.5 + 0.5 * z;
        w[i] = wt;
        w[n - 1 - i] = wt;
    }
}

ScalingBasis::ScalingBasis(int t, int k) : type(t), order(k), K(k + 1) {
    if (t != Legendre && t != Interpol) throw Error(1, "invalid scaling type");
    gauss_legendre01(K, roots, weights);
    vcMap = Mat(K, K);
    if (type == Legendre) {
        for (int i = 0; i < K; i++)
            for (int j = 0; j < K; j++) vcMap(i, j) = legendre_scaled(j, roots[i]) * weights[i];
        cvMap = inverse(vcMap);
    } else {
        cvMap = Mat(K, K);
        for (int i = 0; i < K; i++) {
            cvMap(i, i) = std::sqrt(1.0 / weights[i]);
            vcMap(i, i) = std::sqrt(weights[i]);
        }
    }
    H0 = table(0, type, k);
    G0 = table(1, type, k);
    H1 = Mat(K, K);
    G1 = Mat(K, K);
    for (int i = 0; i < K; i++)
        for (int j = 0; j < K; j++) {
            if (type == Interpol) {
                G1(i, j) = std::pow(-1.0, i + K) * G0(i, K - j - 1);
                H1(i, j) = H0(K - i - 1, K - j - 1);
            } else {
                G1(i, j) = std::pow(-1.0, i + j + K) * G0(i, j);
                H1(i, j) = std::pow(-1.0, i + j) * H0(i, j);
            }
        }
    sub[Compression][0] = H0.transpose();
    sub[Compression][1] = H1.transpose();
    sub[Compression][2] = G0.transpose();
    sub[Compression][3] = G1.transpose();
    sub[Reconstruction][0] = H0;
    sub[Reconstruction][1] = G0;
    sub[Reconstruction][2] = H1;
    sub[Reconstruction][3] = G1;
}

double ScalingBasis::eval(int j, double x) const {
    if (type == Legendre) return legendre_scaled(j, x);
    double s = 0.0;
    for (int m = 0; m < K; m++) s += legendre_scaled(m, roots[j]) * legendre_scaled(m, x);
    return std::sqrt(weights[j]) * s;
}

const ScalingBasis &get_basis(int type, int order) {
    {
        std::lock_guard<std::mutex> lk(g_mu);
        auto it = g_bases.find({type, order});
        if (it != g_bases.end()) return *it->second;
    }
    auto *b = new ScalingBasis(type, order);
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_bases.find({type, order});
    if (it != g_bases.end()) { delete b; return *it->second; }
    g_bases[{type, order}] = b;
    return *b;
}

void apply_filter(double *out, const double *in, const Mat &F, int K, int Kdm1, bool add) {
    // f = in viewed as K x Kdm1 (column-major), g = out viewed as Kdm1 x K
    for (int j = 0; j < K; j++) {
        const double *Fj = F.data() + (size_t)K * j;
        for (int c = 0; c < Kdm1; c++) {
            const double *fc = in + (size_t)K * c;
            double s = 0.0;
            for (int i = 0; i < K; i++) s += fc[i] * Fj[i];
            if (add) out[c + (size_t)Kdm1 * j] += s;
            else out[c + (size_t)Kdm1 * j] = s;
        }
    }
}

template <int D> BoundingBox<D> BoundingBox<D>::fromBounds(int lb, int ub) {
    if (ub < 1) throw Error(1, "Invalid upper bound");
    if (!(lb == 0 || lb == -ub)) throw Error(1, "Invalid lower bound");
    int n = 0;
    double size = 1.0 * ub;
    while (size >= 2.0) { size /= 2.0; n--; }
    BoundingBox<D> b;
    b.scale = n;
    b.corner.fill(lb == 0 ? 0 : -1);
    b.nbox.fill(lb == 0 ? 1 : 2);
    b.sf.fill(size);
    return b;
}
template struct BoundingBox<1>;
template struct BoundingBox<2>;
template struct BoundingBox<3>;

}  // namespace mwh
