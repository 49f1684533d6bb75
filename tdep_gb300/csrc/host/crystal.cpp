// Crystal structure input, masses and space-group operations.
#include "crystal.hpp"

#include <algorithm>
#include <fstream>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <map>
#include <sstream>

namespace tdg {

namespace {

// Standard atomic weights (amu) of the elements the synthetic workloads and the
// reference's test fixtures use. Other elements need infile.isotopes.
const std::map<std::string, double> &atomic_weights() {
    static const std::map<std::string, double> w = {
        {"H", 1.008},     {"Li", 6.94},     {"Be", 9.0122},  {"B", 10.81},    {"C", 12.011},
        {"N", 14.007},    {"O", 15.999},    {"F", 18.998},   {"Na", 22.990},  {"Mg", 24.305},
        {"Al", 26.982},   {"Si", 28.085},   {"P", 30.974},   {"S", 32.06},    {"Cl", 35.45},
        {"K", 39.098},    {"Ca", 40.078},   {"Sc", 44.956},  {"Ti", 47.867},  {"V", 50.942},
        {"Cr", 51.996},   {"Mn", 54.938},   {"Fe", 55.845},  {"Co", 58.933},  {"Ni", 58.693},
        {"Cu", 63.546},   {"Zn", 65.38},    {"Ga", 69.723},  {"Ge", 72.630},  {"As", 74.922},
        {"Se", 78.971},   {"Br", 79.904},   {"Rb", 85.468},  {"Sr", 87.62},   {"Y", 88.906},
        {"Zr", 91.224},   {"Nb", 92.906},   {"Mo", 95.95},   {"Ag", 107.87},  {"Cd", 112.41},
        {"In", 114.82},   {"Sn", 118.71},   {"Sb", 121.76},  {"Te", 127.60},  {"I", 126.90},
        {"Cs", 132.91},   {"Ba", 137.33},   {"La", 138.91},  {"Hf", 178.49},  {"Ta", 180.95},
        {"W", 183.84},    {"Pt", 195.08},   {"Au", 196.97},  {"Pb", 207.2},   {"Bi", 208.98},
    };
    return w;
}

// Natural isotope distributions (abundance, mass in amu): the NIST isotopic compositions
// and relative atomic masses, the public data the reference also tabulates for every
// element (type_crystalstructure.f90:1522, naturaldistribution). As in the reference
// (type_crystalstructure.f90:645-656, 1505-1519), an atom without infile.isotopes takes the
// mean mass of its element's distribution and the mass-disorder parameter
// sum_i c_i (m_i - <m>)^2 / <m>^2 that isotope scattering uses. An element outside this
// table gets its standard atomic weight and an unknown disorder (NaN): isotope scattering
// then stops with an error instead of silently using zero (give infile.isotopes or switch
// isotope scattering off).
using IsoTable = std::map<std::string, std::vector<std::pair<double, double>>>;
const IsoTable &natural_isotopes() {
    static const IsoTable t = {
        {"H", {{0.999885, 1.00782503207}, {0.000115, 2.0141017778}}},
        {"Li", {{0.0759, 6.015122795}, {0.9241, 7.01600455}}},
        {"Be", {{1.0, 9.0121822}}},
        {"B", {{0.199, 10.0129370}, {0.801, 11.0093054}}},
        {"C", {{0.9893, 12.0}, {0.0107, 13.0033548378}}},
        {"N", {{0.99636, 14.0030740048}, {0.00364, 15.0001088982}}},
        {"O", {{0.99757, 15.99491461956}, {0.00038, 16.9991317}, {0.00205, 17.999161}}},
        {"F", {{1.0, 18.99840322}}},
        {"Na", {{1.0, 22.9897692809}}},
        {"Mg", {{0.7899, 23.9850417}, {0.1000, 24.98583692}, {0.1101, 25.982592929}}},
        {"Al", {{1.0, 26.98153863}}},
        {"Si", {{0.92223, 27.9769265325}, {0.04685, 28.976494700}, {0.03092, 29.97377017}}},
        {"P", {{1.0, 30.97376163}}},
        {"S", {{0.9499, 31.97207100}, {0.0075, 32.97145876}, {0.0425, 33.96786690}, {0.0001, 35.96708076}}},
        {"Cl", {{0.7576, 34.96885268}, {0.2424, 36.96590259}}},
        {"K", {{0.932581, 38.96370668}, {0.000117, 39.96399848}, {0.067302, 40.96182576}}},
        {"Ca", {{0.96941, 39.96259098}, {0.00647, 41.95861801}, {0.00135, 42.9587666}, {0.02086, 43.9554818},
                {0.00004, 45.9536926}, {0.00187, 47.952534}}},
        {"Sc", {{1.0, 44.9559119}}},
        {"Ti", {{0.0825, 45.9526316}, {0.0744, 46.9517631}, {0.7372, 47.9479463}, {0.0541, 48.9478700},
                {0.0518, 49.9447912}}},
        {"V", {{0.00250, 49.9471585}, {0.99750, 50.9439595}}},
        {"Cr", {{0.04345, 49.9460442}, {0.83789, 51.9405075}, {0.09501, 52.9406494}, {0.02365, 53.9388804}}},
        {"Mn", {{1.0, 54.9380451}}},
        {"Fe", {{0.05845, 53.9396105}, {0.91754, 55.9349375}, {0.02119, 56.9353940}, {0.00282, 57.9332756}}},
        {"Co", {{1.0, 58.9331950}}},
        {"Ni", {{0.680769, 57.9353429}, {0.262231, 59.9307864}, {0.011399, 60.9310560}, {0.036345, 61.9283451},
                {0.009256, 63.9279660}}},
        {"Cu", {{0.6915, 62.9295975}, {0.3085, 64.9277895}}},
        {"Zn", {{0.48268, 63.9291422}, {0.27975, 65.9260334}, {0.04102, 66.9271273}, {0.19024, 67.9248442},
                {0.00631, 69.9253193}}},
        {"Ga", {{0.60108, 68.9255736}, {0.39892, 70.9247013}}},
        {"Ge", {{0.2038, 69.9242474}, {0.2731, 71.9220758}, {0.0776, 72.9234589}, {0.3672, 73.9211778},
                {0.0783, 75.9214026}}},
        {"As", {{1.0, 74.9215965}}},
        {"Se", {{0.0089, 73.9224764}, {0.0937, 75.9192136}, {0.0763, 76.9199140}, {0.2377, 77.9173091},
                {0.4961, 79.9165213}, {0.0873, 81.9166994}}},
        {"Br", {{0.5069, 78.9183371}, {0.4931, 80.9162906}}},
        {"Sr", {{0.0056, 83.913425}, {0.0986, 85.9092602}, {0.0700, 86.9088771}, {0.8258, 87.9056121}}},
        {"Y", {{1.0, 88.9058483}}},
        {"Zr", {{0.5145, 89.9047044}, {0.1122, 90.9056458}, {0.1715, 91.9050408}, {0.1738, 93.9063152},
                {0.0280, 95.9082734}}},
        {"Nb", {{1.0, 92.9063781}}},
        {"Ag", {{0.51839, 106.905097}, {0.48161, 108.904752}}},
        {"In", {{0.0429, 112.904058}, {0.9571, 114.903878}}},
        {"Sb", {{0.5721, 120.9038157}, {0.4279, 122.9042140}}},
        {"Te", {{0.0009, 119.904020}, {0.0255, 121.9030439}, {0.0089, 122.9042700}, {0.0474, 123.9028179},
                {0.0707, 124.9044307}, {0.1884, 125.9033117}, {0.3174, 127.9044631}, {0.3408, 129.9062244}}},
        {"I", {{1.0, 126.904473}}},
        {"Cs", {{1.0, 132.905451933}}},
        {"Ba", {{0.00106, 129.9063208}, {0.00101, 131.9050613}, {0.02417, 133.9045084}, {0.06592, 134.9056886},
                {0.07854, 135.9045759}, {0.11232, 136.9058274}, {0.71698, 137.9052472}}},
        {"Au", {{1.0, 196.9665687}}},
        {"Pb", {{0.014, 203.9730436}, {0.241, 205.9744653}, {0.221, 206.9758969}, {0.524, 207.9766521}}},
        {"Bi", {{1.0, 208.9803987}}},
    };
    return t;
}

std::vector<std::string> split_ws(const std::string &s) {
    std::istringstream is(s);
    std::vector<std::string> out;
    std::string t;
    while (is >> t) out.push_back(t);
    return out;
}

bool getline_nonempty(std::istream &is, std::string &line) {
    while (std::getline(is, line)) {
        if (line.find_first_not_of(" \t\r") != std::string::npos) return true;
    }
    return false;
}

// A text file in memory, handed out line by line (the force-constant files run to tens of
// thousands of lines; a stream, a string per line and a library conversion per number made
// them the slowest part of a problem load).
class TextFile {
  public:
    bool open(const std::string &path) {
        std::FILE *f = std::fopen(path.c_str(), "rb");
        if (!f) return false;
        bool ok = std::fseek(f, 0, SEEK_END) == 0;
        const long n = ok ? std::ftell(f) : -1;
        ok = n >= 0 && std::fseek(f, 0, SEEK_SET) == 0;
        if (ok) {
            buf_.assign((size_t)n + 1, '\0');
            ok = n == 0 || std::fread(buf_.data(), 1, (size_t)n, f) == (size_t)n;
        }
        std::fclose(f);
        pos_ = 0;
        return ok;
    }
    // The next line with a non-blank character (its start; the line ends at a line break or
    // at the terminating NUL); false at the end of the file.
    bool next(const char *&line) {
        const size_t n = buf_.size() - 1;
        while (pos_ < n) {
            const char *s = buf_.data() + pos_;
            const char *nl = static_cast<const char *>(std::memchr(s, '\n', n - pos_));
            const char *t = nl ? nl : buf_.data() + n;
            pos_ = (size_t)(t - buf_.data()) + (nl ? 1 : 0);
            for (const char *q = s; q < t; ++q)
                if (*q != ' ' && *q != '\t' && *q != '\r') {
                    line = s;
                    return true;
                }
        }
        return false;
    }

  private:
    std::vector<char> buf_;
    size_t pos_ = 0;
};

}  // namespace

int read_poscar(const std::string &path, Crystal &c) {
    std::ifstream f(path);
    if (!f) return set_error(kErrIo, "cannot open " + path);
    std::string line;
    std::getline(f, line);  // header
    if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated " + path);
    const double latpar = std::stod(split_ws(line).at(0));
    M3 m;
    for (int j = 0; j < 3; ++j) {
        if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated " + path);
        auto t = split_ws(line);
        if (t.size() < 3) return set_error(kErrIo, "bad lattice line in " + path);
        for (int i = 0; i < 3; ++i) m(i, j) = std::stod(t[i]);
    }
    if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated " + path);
    c.symbols = split_ws(line);
    if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated " + path);
    auto counts = split_ws(line);
    if (counts.size() != c.symbols.size()) return set_error(kErrIo, "species/count mismatch in " + path);
    if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated " + path);
    char mode = line[line.find_first_not_of(" \t")];
    if (mode == 's' || mode == 'S') {
        if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated " + path);
        mode = line[line.find_first_not_of(" \t")];
    }
    bool cartesian;
    if (mode == 'C' || mode == 'c')
        cartesian = true;
    else if (mode == 'D' || mode == 'd')
        cartesian = false;
    else
        return set_error(kErrIo, "Specify either Cartesian or direct coordinates in " + path);
    // Lattice parameter scales the lattice (negative = volume, as in VASP).
    double scale = latpar;
    if (latpar < 0) scale = std::cbrt(-latpar / std::fabs(det(m)));
    for (double &x : m.a) x *= scale * kAToBohr;
    c.lat = m;
    c.inv_lat = inverse(m);
    c.reclat = transpose(c.inv_lat);  // b_j: columns of A^{-T}
    c.inv_reclat = inverse(c.reclat);
    c.volume = std::fabs(det(m));
    c.frac.clear();
    c.species.clear();
    for (size_t s = 0; s < counts.size(); ++s) {
        const int cnt = std::stoi(counts[s]);
        for (int k = 0; k < cnt; ++k) {
            if (!getline_nonempty(f, line)) return set_error(kErrIo, "truncated positions in " + path);
            auto t = split_ws(line);
            if (t.size() < 3) return set_error(kErrIo, "bad position line in " + path);
            V3 v;
            for (int i = 0; i < 3; ++i) v[i] = std::stod(t[i]);
            if (cartesian) {
                for (int i = 0; i < 3; ++i) v[i] *= scale * kAToBohr;
                v = mul(c.inv_lat, v);
            }
            c.frac.push_back(v);
            c.species.push_back((int)s);
        }
    }
    c.na = (int)c.frac.size();
    c.rcart.resize(c.na);
    c.mass.assign(c.na, 0.0);
    c.invsqrtmass.assign(c.na, 0.0);
    c.disorder.assign(c.na, 0.0);
    for (int a = 0; a < c.na; ++a) {
        c.rcart[a] = c.frac_to_cart(c.frac[a]);
        const auto &nat = natural_isotopes();
        auto nt = nat.find(c.symbols[c.species[a]]);
        if (nt != nat.end()) {
            double mean = 0, g = 0;
            for (const auto &ci : nt->second) mean += ci.first * ci.second * kAmuToEmu;
            for (const auto &ci : nt->second) {
                const double dm = ci.second * kAmuToEmu - mean;
                g += ci.first * dm * dm;
            }
            c.mass[a] = mean;
            c.invsqrtmass[a] = 1.0 / std::sqrt(mean);
            c.disorder[a] = g / (mean * mean);
            continue;
        }
        const auto &w = atomic_weights();
        auto it = w.find(c.symbols[c.species[a]]);
        if (it != w.end()) {
            c.mass[a] = it->second * kAmuToEmu;
            c.invsqrtmass[a] = 1.0 / std::sqrt(c.mass[a]);
        }
        // no natural distribution: the disorder is unknown until infile.isotopes gives it
        c.disorder[a] = std::numeric_limits<double>::quiet_NaN();
    }
    return kOk;
}

int read_isotopes(const std::string &path, Crystal &c) {
    std::ifstream f(path);
    if (!f) return set_error(kErrIo, "cannot open " + path);
    for (int a = 0; a < c.na; ++a) {
        int n = 0;
        if (!(f >> n) || n < 1) return set_error(kErrIo, "bad isotope count in " + path);
        std::vector<double> conc(n), mass(n);
        double csum = 0;
        for (int j = 0; j < n; ++j) {
            if (!(f >> conc[j] >> mass[j])) return set_error(kErrIo, "truncated " + path);
            mass[j] *= kAmuToEmu;
            csum += conc[j];
        }
        double mean = 0;
        for (int j = 0; j < n; ++j) {
            conc[j] /= csum;
            mean += conc[j] * mass[j];
        }
        double g = 0;
        for (int j = 0; j < n; ++j) g += conc[j] * (mass[j] - mean) * (mass[j] - mean);
        c.mass[a] = mean;
        c.invsqrtmass[a] = 1.0 / std::sqrt(mean);
        c.disorder[a] = g / (mean * mean);
    }
    return kOk;
}

namespace {
// Distance of a fractional vector to the nearest lattice point, in Bohr.
double frac_dist(const Crystal &c, const V3 &d) {
    V3 w;
    for (int i = 0; i < 3; ++i) w[i] = d[i] - anint(d[i]);
    return std::sqrt(sqnorm(c.frac_to_cart(w)));
}
}  // namespace

int find_symmetry(Crystal &c) {
    // Metric tensor G = A^T A; a lattice rotation W (integer, fractional) keeps it.
    const M3 G = mul(transpose(c.lat), c.lat);
    double gscale = 0;
    for (double x : G.a) gscale = std::max(gscale, std::fabs(x));
    std::vector<SymOp> ops;
    int w[9];
    for (int code = 0; code < 19683; ++code) {
        int r = code;
        for (int k = 0; k < 9; ++k) {
            w[k] = r % 3 - 1;
            r /= 3;
        }
        M3 W;
        for (int k = 0; k < 9; ++k) W.a[k] = w[k];
        const double d = det(W);
        if (std::fabs(std::fabs(d) - 1.0) > 1e-8) continue;
        const M3 GW = mul(mul(transpose(W), G), W);
        bool ok = true;
        for (int k = 0; k < 9 && ok; ++k) ok = std::fabs(GW.a[k] - G.a[k]) < 1e-6 * gscale;
        if (!ok) continue;
        // Candidate translations map atom 0 onto any atom of the same species.
        for (int j = 0; j < c.na; ++j) {
            if (c.species[j] != c.species[0]) continue;
            const V3 w0 = mul(W, c.frac[0]);
            V3 t;
            for (int i = 0; i < 3; ++i) t[i] = c.frac[j][i] - w0[i];
            for (int i = 0; i < 3; ++i) t[i] -= std::floor(t[i] + 1e-9);
            bool maps = true;
            for (int a = 0; a < c.na && maps; ++a) {
                const V3 wa = mul(W, c.frac[a]);
                bool found = false;
                for (int b = 0; b < c.na && !found; ++b) {
                    if (c.species[b] != c.species[a]) continue;
                    V3 dd;
                    for (int i = 0; i < 3; ++i) dd[i] = wa[i] + t[i] - c.frac[b][i];
                    found = frac_dist(c, dd) < 1e-4;
                }
                maps = found;
            }
            if (!maps) continue;
            SymOp op;
            for (int k = 0; k < 9; ++k) op.fm[k] = w[k];
            op.m = mul(mul(c.lat, W), c.inv_lat);
            // reciprocal fractional rotation: B^-1 m B = W^{-T}
            const M3 rf = transpose(inverse(W));
            for (int k = 0; k < 9; ++k) op.rfm[k] = (int32_t)anint(rf.a[k]);
            op.tr = t;
            ops.push_back(op);
        }
    }
    // Identity (with zero translation) first, the rest in enumeration order.
    auto is_identity = [](const SymOp &o) {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j)
                if (o.fm[i + 3 * j] != (i == j ? 1 : 0)) return false;
        return true;
    };
    std::stable_partition(ops.begin(), ops.end(), is_identity);
    if (ops.empty() || !is_identity(ops[0])) return set_error(kErrSymmetry, "identity operation not found");
    c.ops = ops;
    return kOk;
}

bool parse_real(const char *p, const char **end, double *x) {
    static const double kPow10[23] = {1e0,  1e1,  1e2,  1e3,  1e4,  1e5,  1e6,  1e7,  1e8,  1e9,  1e10, 1e11,
                                      1e12, 1e13, 1e14, 1e15, 1e16, 1e17, 1e18, 1e19, 1e20, 1e21, 1e22};
    static const uint64_t kPow10u[19] = {1ull,
                                         10ull,
                                         100ull,
                                         1000ull,
                                         10000ull,
                                         100000ull,
                                         1000000ull,
                                         10000000ull,
                                         100000000ull,
                                         1000000000ull,
                                         10000000000ull,
                                         100000000000ull,
                                         1000000000000ull,
                                         10000000000000ull,
                                         100000000000000ull,
                                         1000000000000000ull,
                                         10000000000000000ull,
                                         100000000000000000ull,
                                         1000000000000000000ull};
    const char *s = p;
    while (*s == ' ' || *s == '\t') ++s;
    const char *start = s;
    bool neg = false;
    if (*s == '+' || *s == '-') {
        neg = *s == '-';
        ++s;
    }
    // m: up to 19 significant digits, value m 10^e10; tz: trailing zeros of m
    uint64_t m = 0;
    int e10 = 0, nd = 0, tz = 0;
    bool any = false, exact = !(s[0] == '0' && (s[1] == 'x' || s[1] == 'X'));  // hexadecimal: strtod
    for (; exact && *s >= '0' && *s <= '9'; ++s) {
        any = true;
        const int d = *s - '0';
        if (nd < 19) {
            m = m * 10 + (uint64_t)d;
            if (m) ++nd;
            tz = d ? 0 : tz + 1;
        } else {
            ++e10;
            if (d) exact = false;
        }
    }
    if (*s == '.') {
        ++s;
        for (; *s >= '0' && *s <= '9'; ++s) {
            any = true;
            const int d = *s - '0';
            if (nd < 19) {
                m = m * 10 + (uint64_t)d;
                if (m) ++nd;
                tz = d ? 0 : tz + 1;
                --e10;
            } else if (d) {
                exact = false;
            }
        }
    }
    if (any && (*s == 'e' || *s == 'E')) {
        const char *q = s + 1;
        bool en = false;
        if (*q == '+' || *q == '-') {
            en = *q == '-';
            ++q;
        }
        if (*q >= '0' && *q <= '9') {
            int ev = 0;
            for (; *q >= '0' && *q <= '9'; ++q)
                if (ev < 100000) ev = ev * 10 + (*q - '0');
            e10 += en ? -ev : ev;
            s = q;
        }
    }
    if (any && exact) {
        if (m == 0) {
            *x = neg ? -0.0 : 0.0;
            *end = s;
            return true;
        }
        if (tz > 0) {
            m /= kPow10u[tz];
            e10 += tz;
        }
        if (m <= (uint64_t(1) << 53) && e10 >= -22 && e10 <= 22) {
            const double v = (double)m;
            *x = e10 < 0 ? v / kPow10[-e10] : v * kPow10[e10];
            if (neg) *x = -*x;
            *end = s;
            return true;
        }
    }
    char *q = nullptr;
    *x = std::strtod(start, &q);
    *end = q;
    return q != start;
}

namespace {
// The first integer / the first k reals of the next non-empty line, parsed in place. 0 when
// the line is missing or does not start with the numbers.
int read_int_line(TextFile &f, int &x) {
    const char *p = nullptr;
    if (!f.next(p)) return 0;
    char *end = nullptr;
    const long v = std::strtol(p, &end, 10);
    if (end == p) return 0;
    x = (int)v;
    return 1;
}
int read_reals_line(TextFile &f, int k, double *x) {
    const char *p = nullptr;
    if (!f.next(p)) return 0;
    for (int i = 0; i < k; ++i) {
        const char *end = nullptr;
        if (!parse_real(p, &end, x + i)) return 0;
        p = end;
    }
    return 1;
}
int read_vec_line(TextFile &f, double *x) { return read_reals_line(f, 3, x); }
// A force-constant lattice vector must be integer in fractional coordinates.
int to_lattice(const double *x, int32_t *out) {
    for (int i = 0; i < 3; ++i) {
        const double r = anint(x[i]);
        if (std::fabs(x[i] - r) > 1e-6) return 0;
        out[i] = (int32_t)r;
    }
    return 1;
}
}  // namespace

int read_fc2(const std::string &path, const Crystal &c, FC2 &fc) {
    TextFile f;
    if (!f.open(path)) return set_error(kErrIo, "cannot open " + path);
    auto first_tokens = [&](int k, std::vector<double> &out) -> bool {
        out.resize(k);
        return read_reals_line(f, k, out.data()) != 0;
    };
    std::vector<double> v;
    if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);
    fc.na = (int)v[0];
    if (fc.na != c.na)
        return set_error(kErrIo, "different number of atoms in \"" + path + "\" and the structure");
    if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);  // cutoff
    fc.pairs.clear();
    for (int a1 = 0; a1 < fc.na; ++a1) {
        if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);
        const int n = (int)v[0];
        for (int i = 0; i < n; ++i) {
            FC2Pair p;
            p.a1 = a1;
            if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);
            p.a2 = (int)v[0] - 1;
            if (p.a2 < 0 || p.a2 >= c.na) return set_error(kErrIo, "bad atom index in " + path);
            if (!first_tokens(3, v)) return set_error(kErrIo, "truncated " + path);
            V3 lvf;
            for (int k = 0; k < 3; ++k) lvf[k] = v[k];
            p.lv = c.frac_to_cart(lvf);
            for (int k = 0; k < 3; ++k)
                if (std::fabs(p.lv[k]) < kSqTol) p.lv[k] = 0.0;
            for (int j = 0; j < 3; ++j) {
                if (!first_tokens(3, v)) return set_error(kErrIo, "truncated " + path);
                for (int k = 0; k < 3; ++k) p.m[j + 3 * k] = v[k] * kFc2EvAToHaBohr;
            }
            fc.pairs.push_back(p);
        }
    }
    // Polar block (type_forceconstant_secondorder_io.f90:172-196).
    fc.polar = 0;
    if (first_tokens(1, v)) fc.polar = (int)v[0];
    if (fc.polar == 0) return kOk;
    if (fc.polar == 1 || fc.polar == 2)
        return set_error(kErrIo, "This polar correction type is deprecated (" + path + ")");
    if (fc.polar != 3) return set_error(kErrIo, "Undefined polar correction type in " + path);
    for (int col = 0; col < 3; ++col) {  // eps(:, col), one line each
        if (!first_tokens(3, v)) return set_error(kErrIo, "truncated " + path);
        for (int r = 0; r < 3; ++r) fc.eps(r, col) = v[r];
    }
    if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);
    fc.lambda = v[0];
    if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);
    const int nx = (int)v[0];
    if (nx < 0) return set_error(kErrIo, "bad number of Born-charge components in " + path);
    std::vector<double> x(nx), coeff((size_t)9 * fc.na * nx);
    for (int i = 0; i < nx; ++i) {
        if (!first_tokens(1, v)) return set_error(kErrIo, "truncated " + path);
        x[i] = v[0];
    }
    for (int r = 0; r < 9 * fc.na; ++r) {
        if (nx > 0 && !first_tokens(nx, v)) return set_error(kErrIo, "truncated " + path);
        for (int i = 0; i < nx; ++i) coeff[(size_t)r * nx + i] = v[i];
    }
    // Zflat = coeff_Z x_Z, unflattened row by row (gottochblandat_tensors.f90:191-203).
    fc.Z.assign((size_t)9 * fc.na, 0.0);
    double tot[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    for (int a = 0; a < fc.na; ++a)
        for (int l = 0; l < 9; ++l) {
            double zf = 0;
            for (int i = 0; i < nx; ++i) zf += coeff[(size_t)(a * 9 + l) * nx + i] * x[i];
            const int i = l / 3, j = l % 3;
            fc.Z[(size_t)a * 9 + i + 3 * j] = zf;
            tot[i + 3 * j] += zf;
        }
    double s = 0;
    for (double t : tot) s += std::fabs(t);
    if (s > kSqTol) return set_error(kErrSymmetry, "Born charges do not add up to zero");

    // Reciprocal vectors of the Ewald sum. The reference fixes the radius by a root search
    // on the Gaussian tail (lo_longrange_electrostatics.f90:392-480, tolerance 1e-20) plus
    // the bounding sphere of the reciprocal cell; this takes every vector whose Gaussian
    // factor exp(-|K|^2_eps / 4 lambda^2) |K|^2_eps can exceed 1e-30, plus the sum of the
    // reciprocal basis lengths, a superset whose extra terms are below that bound.
    std::vector<cplx> em(9);
    for (int i = 0; i < 9; ++i) em[i] = fc.eps.a[i];
    std::vector<double> ew;
    std::vector<cplx> evec;
    int st = hermitian_jacobi(3, em, ew, evec);
    if (st) return st;
    const double emin = std::min({ew[0], ew[1], ew[2]}), emax = std::max({ew[0], ew[1], ew[2]});
    if (!(emin > 0) || !(fc.lambda > 0))
        return set_error(kErrIo, "polar block needs a positive-definite dielectric tensor and lambda > 0");
    const double inv4l2 = 1.0 / (4.0 * fc.lambda * fc.lambda);
    double r0 = 0;
    for (;;) {
        r0 += 1e-3;
        const double kk = kTwoPi * kTwoPi * r0 * r0;
        if (std::exp(-kk * emin * inv4l2) * kk * emax < 1e-30) break;
    }
    double krad = r0;
    for (int i = 0; i < 3; ++i)
        krad += std::sqrt(c.reclat(0, i) * c.reclat(0, i) + c.reclat(1, i) * c.reclat(1, i) +
                          c.reclat(2, i) * c.reclat(2, i));
    int bd[3];
    for (int i = 0; i < 3; ++i) {
        const double al = std::sqrt(c.lat(0, i) * c.lat(0, i) + c.lat(1, i) * c.lat(1, i) + c.lat(2, i) * c.lat(2, i));
        bd[i] = (int)std::ceil(krad * al) + 1;
    }
    std::vector<std::pair<double, V3>> gl;
    for (int i = -bd[0]; i <= bd[0]; ++i)
        for (int j = -bd[1]; j <= bd[1]; ++j)
            for (int k = -bd[2]; k <= bd[2]; ++k) {
                V3 f;
                f[0] = i;
                f[1] = j;
                f[2] = k;
                const V3 g = mul(c.reclat, f);
                const double n2 = sqnorm(g);
                if (n2 < krad * krad) gl.push_back({n2, g});
            }
    // Longest first, as the reference stores them.
    std::stable_sort(gl.begin(), gl.end(), [](const auto &a, const auto &b) { return a.first > b.first; });
    fc.G.clear();
    for (const auto &e : gl) fc.G.push_back(e.second);

    // Onsite correction: minus the row sums of the real long-range matrix at Gamma,
    // chopped at 1e-13 (type_forceconstant_secondorder_loto.f90:76-96).
    fc.Zonsite.assign((size_t)9 * fc.na, 0.0);
    std::vector<cplx> dc((size_t)9 * fc.na * fc.na);
    longrange_dm(c, fc, V3(), false, dc.data(), nullptr);
    double im = 0;
    for (const auto &z : dc) im += std::fabs(z.imag());
    if (im > kSqTol * fc.na * fc.na) return set_error(kErrSymmetry, "Dynamical matrix at gamma not real.");
    for (int a1 = 0; a1 < fc.na; ++a1)
        for (int e = 0; e < 9; ++e) {
            double m = 0;
            for (int a2 = 0; a2 < fc.na; ++a2) m += dc[((size_t)a1 * fc.na + a2) * 9 + e].real();
            fc.Zonsite[(size_t)a1 * 9 + e] = std::fabs(m) < 1e-13 ? 0.0 : -m;
        }
    return kOk;
}


int read_fc3(const std::string &path, const Crystal &c, FC3 &fc) {
    TextFile f;
    if (!f.open(path)) return set_error(kErrIo, "cannot open " + path);
    int na = 0;
    double cut[3];
    if (!read_int_line(f, na)) return set_error(kErrIo, "truncated " + path);
    const char *line = nullptr;
    if (!f.next(line)) return set_error(kErrIo, "truncated " + path);
    (void)cut;
    if (na != c.na) return set_error(kErrIo, "different number of atoms in \"" + path + "\" and the structure");
    fc.atoms.clear();
    fc.lv.clear();
    fc.lvcart.clear();
    fc.mwm.clear();
    for (int a1 = 0; a1 < na; ++a1) {
        int n = 0;
        if (!read_int_line(f, n)) return set_error(kErrIo, "truncated " + path);
        for (int t = 0; t < n; ++t) {
            int ii[3];
            for (int k = 0; k < 3; ++k)
                if (!read_int_line(f, ii[k])) return set_error(kErrIo, "truncated " + path);
            for (int k = 0; k < 3; ++k)
                if (ii[k] < 1 || ii[k] > na) return set_error(kErrIo, "bad atom index in " + path);
            double lvs[9];
            for (int k = 0; k < 3; ++k)
                if (!read_vec_line(f, lvs + 3 * k)) return set_error(kErrIo, "truncated " + path);
            int32_t lvi[9];
            for (int k = 0; k < 3; ++k)
                if (!to_lattice(lvs + 3 * k, lvi + 3 * k))
                    return set_error(kErrIo, "non-integer lattice vector in " + path);
            double m[27];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    double v[3];
                    if (!read_vec_line(f, v)) return set_error(kErrIo, "truncated " + path);
                    for (int k = 0; k < 3; ++k) m[i + 3 * j + 9 * k] = v[k] * kFc3EvAToHaBohr;
                }
            const double w = c.invsqrtmass[ii[0] - 1] * c.invsqrtmass[ii[1] - 1] * c.invsqrtmass[ii[2] - 1];
            for (int k = 0; k < 3; ++k) fc.atoms.push_back(ii[k]);
            for (int k = 3; k < 9; ++k) fc.lv.push_back(lvi[k]);
            for (int k = 1; k < 3; ++k) {
                V3 lf;
                for (int i = 0; i < 3; ++i) lf[i] = lvs[3 * k + i];
                V3 lc = c.frac_to_cart(lf);
                for (int i = 0; i < 3; ++i) fc.lvcart.push_back(std::fabs(lc[i]) < kSqTol ? 0.0 : lc[i]);
            }
            for (int k = 0; k < 27; ++k) fc.mwm.push_back(m[k] * w);
        }
    }
    return kOk;
}

int read_fc4(const std::string &path, const Crystal &c, FC4 &fc) {
    TextFile f;
    if (!f.open(path)) return set_error(kErrIo, "cannot open " + path);
    int na = 0;
    if (!read_int_line(f, na)) return set_error(kErrIo, "truncated " + path);
    const char *line = nullptr;
    if (!f.next(line)) return set_error(kErrIo, "truncated " + path);
    if (na != c.na) return set_error(kErrIo, "different number of atoms in \"" + path + "\" and the structure");
    fc.atoms.clear();
    fc.lv.clear();
    fc.lvcart.clear();
    fc.mwm.clear();
    for (int a1 = 0; a1 < na; ++a1) {
        int n = 0;
        if (!read_int_line(f, n)) return set_error(kErrIo, "truncated " + path);
        for (int t = 0; t < n; ++t) {
            int ii[4];
            for (int k = 0; k < 4; ++k)
                if (!read_int_line(f, ii[k])) return set_error(kErrIo, "truncated " + path);
            for (int k = 0; k < 4; ++k)
                if (ii[k] < 1 || ii[k] > na) return set_error(kErrIo, "bad atom index in " + path);
            double lvs[12];
            for (int k = 0; k < 4; ++k)
                if (!read_vec_line(f, lvs + 3 * k)) return set_error(kErrIo, "truncated " + path);
            int32_t lvi[12];
            for (int k = 0; k < 4; ++k)
                if (!to_lattice(lvs + 3 * k, lvi + 3 * k))
                    return set_error(kErrIo, "non-integer lattice vector in " + path);
            double m[81];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j)
                    for (int k = 0; k < 3; ++k) {
                        double v[3];
                        if (!read_vec_line(f, v)) return set_error(kErrIo, "truncated " + path);
                        for (int l = 0; l < 3; ++l) m[i + 3 * j + 9 * k + 27 * l] = v[l] * kFc4EvAToHaBohr;
                    }
            const double w = c.invsqrtmass[ii[0] - 1] * c.invsqrtmass[ii[1] - 1] *
                             c.invsqrtmass[ii[2] - 1] * c.invsqrtmass[ii[3] - 1];
            for (int k = 0; k < 4; ++k) fc.atoms.push_back(ii[k]);
            for (int k = 3; k < 12; ++k) fc.lv.push_back(lvi[k]);
            for (int k = 1; k < 4; ++k) {
                V3 lf;
                for (int i = 0; i < 3; ++i) lf[i] = lvs[3 * k + i];
                V3 lc = c.frac_to_cart(lf);
                for (int i = 0; i < 3; ++i) fc.lvcart.push_back(std::fabs(lc[i]) < kSqTol ? 0.0 : lc[i]);
            }
            for (int k = 0; k < 81; ++k) fc.mwm.push_back(m[k] * w);
        }
    }
    return kOk;
}

int op_atom_maps(const Crystal &c, std::vector<int32_t> &fmap, std::vector<double> &shift) {
    const int na = c.na, no = (int)c.ops.size();
    fmap.assign((size_t)no * na, -1);
    shift.assign((size_t)no * na * 3, 0.0);
    for (int o = 0; o < no; ++o) {
        const SymOp &op = c.ops[o];
        M3 W;
        for (int k = 0; k < 9; ++k) W.a[k] = op.fm[k];
        const M3 Wi = inverse(W);
        for (int a = 0; a < na; ++a) {
            const V3 img = mul(W, c.frac[a]);
            int hit = -1;
            for (int b = 0; b < na && hit < 0; ++b) {
                if (c.species[b] != c.species[a]) continue;
                V3 d;
                for (int i = 0; i < 3; ++i) d[i] = img[i] + op.tr[i] - c.frac[b][i];
                if (frac_dist(c, d) < 1e-4) hit = b;
            }
            if (hit < 0) return set_error(kErrSymmetry, "an operation does not map the crystal onto itself");
            fmap[(size_t)o * na + a] = hit;
            V3 u;
            for (int i = 0; i < 3; ++i) u[i] = c.frac[hit][i] - op.tr[i];
            V3 v = mul(Wi, u);
            for (int i = 0; i < 3; ++i) v[i] = anint(v[i] - c.frac[a][i]);
            const V3 w = c.frac_to_cart(v);
            for (int i = 0; i < 3; ++i) shift[((size_t)o * na + a) * 3 + i] = w[i];
        }
    }
    return kOk;
}

}  // namespace tdg

extern "C" int tdg_natural_isotopes(const char *symbol, int32_t cap, double *abundance, double *mass) {
    if (!symbol) return tdg::set_error(tdg::kErrParam, "tdg_natural_isotopes: null symbol");
    const auto &t = tdg::natural_isotopes();
    auto it = t.find(symbol);
    if (it == t.end()) return 0;
    const int32_t n = (int32_t)it->second.size();
    if (cap < n || !abundance || !mass) return -n;
    for (int32_t i = 0; i < n; ++i) {
        abundance[i] = it->second[i].first;
        mass[i] = it->second[i].second;
    }
    return n;
}
