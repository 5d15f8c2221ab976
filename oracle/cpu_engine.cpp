// CPU restatement of the Upside ff_2.1 force evaluation (test infrastructure:
// the oracle).  See cpu_engine.h.  Each node cites the reference file:line it
// restates.  Arithmetic is scalar and templated on T (float tracks the
// reference; double is the FP64 yardstick).
#include "cpu_engine.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include "h5lite.h"

namespace {

using std::string;
using std::vector;

thread_local string g_err;

struct Err : std::runtime_error {
    explicit Err(const string& s) : std::runtime_error(s) {}
};

// ------------------------------------------------------------------ math ---
template <class T> struct V3 {
    T x, y, z;
    V3() : x(0), y(0), z(0) {}
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    V3 operator+(const V3& o) const { return {x + o.x, y + o.y, z + o.z}; }
    V3 operator-(const V3& o) const { return {x - o.x, y - o.y, z - o.z}; }
    V3 operator-() const { return {-x, -y, -z}; }
    V3 operator*(T s) const { return {x * s, y * s, z * s}; }
    V3& operator+=(const V3& o) { x += o.x; y += o.y; z += o.z; return *this; }
    V3& operator-=(const V3& o) { x -= o.x; y -= o.y; z -= o.z; return *this; }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};
template <class T> V3<T> operator*(T s, const V3<T>& v) { return v * s; }
template <class T> T dot(const V3<T>& a, const V3<T>& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
template <class T> V3<T> cross(const V3<T>& a, const V3<T>& b) {
    return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
template <class T> T mag2(const V3<T>& a) { return dot(a, a); }
template <class T> V3<T> ld3(const T* p) { return {p[0], p[1], p[2]}; }
template <class T> void add3(T* p, const V3<T>& v) { p[0] += v.x; p[1] += v.y; p[2] += v.z; }
template <class T> void st3(T* p, const V3<T>& v) { p[0] = v.x; p[1] = v.y; p[2] = v.z; }

// value and derivative of the compact sigmoid (src/vector_math.h:702-720)
template <class T> void compact_sigmoid(T x, T s, T& v, T& d) {
    T y = x * s;
    if (y > T(1)) { v = 0; d = 0; return; }
    if (y < T(-1)) { v = 1; d = 0; return; }
    v = T(0.25) * (y + T(2)) * (y - T(1)) * (y - T(1));
    d = (s * T(0.75)) * (y * y - T(1));
}

// logistic sigmoid and derivative (src/vector_math.h:689-695)
template <class T> void sigmoid(T x, T& v, T& d) {
    T z = std::exp(-x);
    T w = T(1) / (T(1) + z);
    v = w;
    d = z * w * w;
}

// Uniform cubic B-spline basis on a unit interval and its derivative.
template <class T> void bspline4(T y, T b[4], T db[4]) {
    T y2 = y * y, y3 = y2 * y, o = T(1) - y;
    b[0] = o * o * o / T(6);
    b[1] = (T(3) * y3 - T(6) * y2 + T(4)) / T(6);
    b[2] = (T(-3) * y3 + T(3) * y2 + T(3) * y + T(1)) / T(6);
    b[3] = y3 / T(6);
    db[0] = -o * o / T(2);
    db[1] = (T(3) * y2 - T(4) * y) / T(2);
    db[2] = (T(-3) * y2 + T(2) * y + T(1)) / T(2);
    db[3] = y2 / T(2);
}

// B-spline value/derivative with the first spline centred at -1
// (deBoor_value_and_deriv, src/spline.h:98-129); requires x >= 1.
template <class T> void deboor(const T* c, T x, T& v, T& d) {
    int xb = int(x);
    T b[4], db[4];
    bspline4(x - T(xb), b, db);
    const T* cc = c + (xb - 1);
    v = cc[0] * b[0] + cc[1] * b[1] + cc[2] * b[2] + cc[3] * b[3];
    d = cc[0] * db[0] + cc[1] * db[1] + cc[2] * db[2] + cc[3] * db[3];
}

// Clamped spline with constant ends (src/spline.h:278-358)
template <class T> void clamped(const T* c, T x, int n, T& v, T& d) {
    if (x <= T(1)) {
        v = c[0] / T(6) + c[1] * (T(2) / T(3)) + c[2] / T(6);
        d = 0;
    } else if (x >= T(n - 2)) {
        v = c[n - 3] / T(6) + c[n - 2] * (T(2) / T(3)) + c[n - 1] / T(6);
        d = 0;
    } else {
        deboor(c, x, v, d);
    }
}

// derivative of a clamped spline value w.r.t. its 4 active coefficients
// (clamped_deBoor_coeff_deriv, src/spline.h:423-440)
template <class T> int clamped_coeff_deriv(T x, int n, T r[4]) {
    if (x <= T(1)) { r[0] = T(1) / 6; r[1] = T(2) / 3; r[2] = T(1) / 6; r[3] = 0; return 0; }
    if (x >= T(n - 2)) { r[0] = 0; r[1] = T(1) / 6; r[2] = T(2) / 3; r[3] = T(1) / 6; return n - 4; }
    int xb = int(x);
    T db[4];
    bspline4(x - T(xb), r, db);
    return xb - 1;
}
template <class T> int coeff_deriv(T x, T r[4]) {
    int xb = int(x);
    T db[4];
    bspline4(x - T(xb), r, db);
    return xb - 1;
}

// Solve the cyclic tridiagonal system (1/6, 2/3, 1/6) c = d in double
// (periodic interpolating cubic B-spline), by the Sherman-Morrison update of
// a plain tridiagonal solve.
void cyclic_bspline_solve(int n, const double* d, double* c) {
    const double a = 1. / 6., b = 2. / 3., cc = 1. / 6.;
    // A = T + u v^T with T tridiagonal(a, b', cc) and corners handled by u,v
    double gamma = -b;
    vector<double> bb(n, b), u(n, 0.), y(d, d + n), z(n), cp(n);
    bb[0] = b - gamma;
    bb[n - 1] = b - a * cc / gamma;
    u[0] = gamma;
    u[n - 1] = cc;
    auto tri = [&](vector<double>& rhs, vector<double>& x) {
        // Thomas algorithm on (a, bb, cc)
        cp[0] = cc / bb[0];
        x[0] = rhs[0] / bb[0];
        for (int i = 1; i < n; ++i) {
            double m = bb[i] - a * cp[i - 1];
            cp[i] = cc / m;
            x[i] = (rhs[i] - a * x[i - 1]) / m;
        }
        for (int i = n - 2; i >= 0; --i) x[i] -= cp[i] * x[i + 1];
    };
    vector<double> ys(n);
    tri(y, ys);
    tri(u, z);
    // v = (1, 0, ..., 0, a/gamma)
    double vy = ys[0] + a / gamma * ys[n - 1];
    double vz = z[0] + a / gamma * z[n - 1];
    double f = vy / (1. + vz);
    for (int i = 0; i < n; ++i) c[i] = ys[i] - f * z[i];
}

// Layered periodic bicubic spline (LayeredPeriodicSpline2D, src/spline.h:444-499),
// held as B-spline coefficients C[layer][x][y].
template <class T> struct Periodic2D {
    int n_layer = 0, nx = 0, ny = 0;
    vector<T> C;
    void fit(int L, int nx_, int ny_, const vector<double>& data) {
        n_layer = L; nx = nx_; ny = ny_;
        C.assign(size_t(L) * nx * ny, T(0));
        vector<double> tmp(size_t(nx) * ny), row(std::max(nx, ny)), out(std::max(nx, ny));
        for (int l = 0; l < L; ++l) {
            const double* dl = data.data() + size_t(l) * nx * ny;
            for (int ix = 0; ix < nx; ++ix) {
                cyclic_bspline_solve(ny, dl + size_t(ix) * ny, out.data());
                for (int iy = 0; iy < ny; ++iy) tmp[size_t(ix) * ny + iy] = out[iy];
            }
            for (int iy = 0; iy < ny; ++iy) {
                for (int ix = 0; ix < nx; ++ix) row[ix] = tmp[size_t(ix) * ny + iy];
                cyclic_bspline_solve(nx, row.data(), out.data());
                for (int ix = 0; ix < nx; ++ix) C[(size_t(l) * nx + ix) * ny + iy] = T(out[ix]);
            }
        }
    }
    void eval(int layer, T x, T y, T& v, T& dx, T& dy) const {
        int xb = int(x), yb = int(y);
        T bx[4], dbx[4], by[4], dby[4];
        bspline4(x - T(xb), bx, dbx);
        bspline4(y - T(yb), by, dby);
        v = dx = dy = 0;
        for (int i = 0; i < 4; ++i) {
            int ix = ((xb - 1 + i) % nx + nx) % nx;
            const T* rowp = C.data() + (size_t(layer) * nx + ix) * ny;
            T sv = 0, sd = 0;
            for (int j = 0; j < 4; ++j) {
                int iy = ((yb - 1 + j) % ny + ny) % ny;
                sv += rowp[iy] * by[j];
                sd += rowp[iy] * dby[j];
            }
            v += bx[i] * sv;
            dx += dbx[i] * sv;
            dy += bx[i] * sd;
        }
    }
};

// quaternion -> rotation matrix (src/affine.h:99-108)
template <class T> void quat_to_rot(const T* q, T* U) {
    T a = q[0], b = q[1], c = q[2], d = q[3];
    U[0] = a * a + b * b - c * c - d * d; U[1] = 2 * b * c - 2 * a * d; U[2] = 2 * b * d + 2 * a * c;
    U[3] = 2 * b * c + 2 * a * d; U[4] = a * a - b * b + c * c - d * d; U[5] = 2 * c * d - 2 * a * b;
    U[6] = 2 * b * d - 2 * a * c; U[7] = 2 * c * d + 2 * a * b; U[8] = a * a - b * b - c * c + d * d;
}
template <class T> V3<T> rot(const T* U, const V3<T>& r) {
    return {U[0] * r.x + U[1] * r.y + U[2] * r.z, U[3] * r.x + U[4] * r.y + U[5] * r.z,
            U[6] * r.x + U[7] * r.y + U[8] * r.z};
}
template <class T> V3<T> rot_inv(const T* U, const V3<T>& r) {
    return {U[0] * r.x + U[3] * r.y + U[6] * r.z, U[1] * r.x + U[4] * r.y + U[7] * r.z,
            U[2] * r.x + U[5] * r.y + U[8] * r.z};
}

// Symmetric 4x4 eigen-decomposition as the reference's AffineAlignment does it
// (src/eig.cpp:57-275): Householder tridiagonalisation (Golub & van Loan 8.3.1),
// then implicit symmetric QR steps with a Wilkinson shift (G&vL 8.3.2-8.3.3),
// off-diagonals zeroed once |u_i| <= 1e-5 (|d_i| + |d_i+1|).  The reference
// runs four consecutive residues through it as one SIMD group, so the
// choice of the active block (and the end of the iteration) is made jointly:
// a block is worked while ANY lane of the group still has a nonzero
// off-diagonal there.  nl lanes (1..4) are given; evals[l*4+k] and
// evec[l*16+k*4+i] (eigenvector k, component i) come back with the largest
// eigenvalue swapped into slot 0 (src/eig.cpp:355-372), others unsorted.
// Packed upper triangle: row i holds A(i,i..3).
static inline int tri4(int i, int j) {
    if (i > j) std::swap(i, j);
    static const int row0[4] = {0, 4, 7, 9};
    return row0[i] + (j - i);
}
template <class T> void qr4_group(int nl, const T (*F)[4][4], T* evals, T* evec) {
    const T tol = T(1e-5), tiny = T(1e-20);
    T A[4][10], d[4][4], u[4][3], Q[4][4][4], beta[4][2];
    for (int l = 0; l < nl; ++l) {
        for (int i = 0; i < 4; ++i)
            for (int j = i; j < 4; ++j) A[l][tri4(i, j)] = F[l][i][j];
        // two Householder reflections reduce A to tridiagonal form; each
        // reflection vector v (v_0 = 1) is kept in place of the column
        for (int k = 0; k < 2; ++k) {
            const int m = 3 - k;
            T* x = &A[l][tri4(k, k + 1)];  // the m entries A(k, k+1..3) are contiguous
            T sig = tiny;
            for (int i = 1; i < m; ++i) sig += x[i] * x[i];
            T mu = std::sqrt(x[0] * x[0] + sig);
            T s = x[0] > T(0) ? -sig / (x[0] + mu) : x[0] - mu;
            T b = T(2) * s * s / (sig + s * s);
            x[0] = mu;
            for (int i = 1; i < m; ++i) x[i] /= s;
            beta[l][k] = b;
            auto v = [&](int j) { return j == 0 ? T(1) : A[l][tri4(k, k + 1 + j)]; };
            T p[3], w[3], pv = 0;
            for (int i = 0; i < m; ++i) {
                p[i] = 0;
                for (int j = 0; j < m; ++j) p[i] += A[l][tri4(i + k + 1, j + k + 1)] * v(j);
                p[i] *= b;
            }
            for (int i = 0; i < m; ++i) pv += p[i] * v(i);
            for (int i = 0; i < m; ++i) w[i] = p[i] - (T(0.5) * b * pv) * v(i);
            for (int i = 0; i < m; ++i)
                for (int j = i; j < m; ++j) A[l][tri4(i + k + 1, j + k + 1)] -= v(i) * w[j] + v(j) * w[i];
        }
        for (int i = 0; i < 4; ++i) d[l][i] = A[l][tri4(i, i)];
        for (int i = 0; i < 3; ++i) u[l][i] = A[l][tri4(i, i + 1)];
        // accumulated orthogonal factor H0 H1 (rows become eigenvectors)
        auto v0 = [&](int j) { return j == 0 ? T(1) : A[l][tri4(0, 1 + j)]; };
        auto v1 = [&](int j) { return j == 0 ? T(1) : A[l][tri4(1, 2 + j)]; };
        T (*R)[4] = Q[l];
        for (int i = 0; i < 4; ++i)
            for (int j = i; j < 4; ++j) R[i][j] = (i == j) ? T(1) : T(0);
        for (int i = 1; i < 4; ++i)
            for (int j = i; j < 4; ++j) R[i][j] -= beta[l][0] * (v0(i - 1) * v0(j - 1));
        for (int i = 2; i < 4; ++i)
            for (int j = i; j < 4; ++j) R[i][j] -= beta[l][1] * (v1(i - 2) * v1(j - 2));
        for (int i = 0; i < 4; ++i)
            for (int j = i + 1; j < 4; ++j) R[j][i] = R[i][j];
        T cpl = beta[l][0] * beta[l][1] * (v0(1) * v1(0) + v0(2) * v1(1));
        for (int i = 2; i < 4; ++i)
            for (int j = 1; j < 4; ++j) R[i][j] += cpl * v1(i - 2) * v0(j - 1);
    }
    for (int it = 0; it < 100; ++it) {
        bool nz[3] = {false, false, false};
        for (int l = 0; l < nl; ++l)
            for (int i = 0; i < 3; ++i) {
                if (std::fabs(u[l][i]) <= tol * (std::fabs(d[l][i]) + std::fabs(d[l][i + 1]))) u[l][i] = 0;
                nz[i] = nz[i] || u[l][i] != T(0);
            }
        int q = nz[2] ? 0 : nz[1] ? 1 : nz[0] ? 2 : 3;
        if (q == 3) break;
        int p = 3 - q;
        for (; p > 0; --p)
            if (!nz[p - 1]) break;
        const int n = 4 - q - p;
        for (int l = 0; l < nl; ++l) {
            T* dd = d[l] + p;
            T* uu = u[l] + p;
            T dv = T(0.5) * (dd[n - 2] - dd[n - 1]) + tiny;
            T un = uu[n - 2];
            T mu = dd[n - 1] - un * un / (dv + std::copysign(std::sqrt(dv * dv + un * un), dv));
            T x = dd[0] - mu, z = uu[0];
            for (int k = 0; k < n - 1; ++k) {
                T c = 1, s = 0;
                if (z != T(0)) {
                    T ir = T(1) / std::sqrt(x * x + z * z);
                    c = x * ir;
                    s = -z * ir;
                }
                for (int j = 0; j < 4; ++j) {
                    T t1 = Q[l][p + k][j], t2 = Q[l][p + k + 1][j];
                    Q[l][p + k][j] = c * t1 - s * t2;
                    Q[l][p + k + 1][j] = s * t1 + c * t2;
                }
                if (k > 0) uu[k - 1] = c * x - s * z;
                T a00 = dd[k], a11 = dd[k + 1], a01 = uu[k];
                dd[k] = a00 * c * c - a01 * T(2) * c * s + a11 * s * s;
                dd[k + 1] = a00 * s * s + a01 * T(2) * c * s + a11 * c * c;
                uu[k] = (a00 - a11) * c * s + a01 * (c * c - s * s);
                x = uu[k];
                if (k < n - 2) {
                    z = -uu[k + 1] * s;
                    uu[k + 1] *= c;
                }
            }
        }
    }
    for (int l = 0; l < nl; ++l) {
        T* ev = evals + 4 * l;
        T* vc = evec + 16 * l;
        for (int k = 0; k < 4; ++k) {
            ev[k] = d[l][k];
            for (int i = 0; i < 4; ++i) vc[4 * k + i] = Q[l][k][i];
        }
        for (int k = 1; k < 4; ++k)
            if (ev[0] < ev[k]) {
                std::swap(ev[0], ev[k]);
                for (int i = 0; i < 4; ++i) std::swap(vc[i], vc[4 * k + i]);
            }
    }
}

// ------------------------------------------------------------- h5 helpers --
struct H5 {
    h5lite::File& f;
    string g;
    string p(const string& n) const { return g + "/" + n; }
    bool has(const string& n) const { return f.exists(p(n)); }
    vector<int> ri(const string& n) const {
        auto v = f.read<int32_t>(p(n));
        return vector<int>(v.begin(), v.end());
    }
    template <class T> vector<T> rf(const string& n) const {
        if (std::is_same<T, float>::value) {
            auto v = f.read<float>(p(n));
            return vector<T>(v.begin(), v.end());
        }
        auto v = f.read<double>(p(n));
        return vector<T>(v.begin(), v.end());
    }
    vector<double> rd(const string& n) const { return f.read<double>(p(n)); }
    vector<uint64_t> dims(const string& n) const { return f.dims(p(n)); }
    bool has_attr(const string& obj, const string& a) const {
        string q = obj.empty() ? g : p(obj);
        return f.has_attr(q, a);
    }
    double attr(const string& a, double def = NAN, const string& obj = "") const {
        string q = obj.empty() ? g : p(obj);
        if (!f.has_attr(q, a)) {
            if (std::isnan(def)) throw Err("missing attribute " + a + " on " + q);
            return def;
        }
        return f.attr_values<double>(q, a).at(0);
    }
};

template <class T> T fcast(double x) { return T(x); }

// ---------------------------------------------------------------- engine ---
template <class T> struct Engine;

template <class T> struct Node {
    string name;
    vector<int> args;
    bool potential_node = false;
    int n_elem = 0, width = 0;
    vector<T> out, sens;
    T pot = 0;
    virtual ~Node() {}
    void alloc(int n, int w) {
        n_elem = n;
        width = w;
        out.assign(size_t(n) * w, T(0));
        sens.assign(size_t(n) * w, T(0));
    }
    virtual void forward(Engine<T>& e, bool energy) = 0;
    virtual void backward(Engine<T>&) {}
    virtual vector<float> value_by_name(const string& w) { throw Err("value '" + w + "' not implemented"); }
    virtual vector<float> get_param() { return {}; }
    virtual void set_param(const vector<float>&) { throw Err("set_param not supported"); }
    virtual vector<float> param_deriv(Engine<T>&) { return {}; }
    virtual const vector<std::pair<int, int>>* edges() const { return nullptr; }
};

template <class T> struct Engine {
    vector<std::unique_ptr<Node<T>>> nodes;  // topological order, nodes[0] = pos
    std::map<string, int> index;
    double potential = 0;
    Node<T>& arg(const Node<T>& n, int i) { return *nodes[size_t(n.args.at(size_t(i)))]; }
    void compute(bool energy) {
        potential = 0;
        for (auto& n : nodes) {
            n->forward(*this, energy);
            if (n->potential_node) {
                if (energy) potential += double(n->pot);
            } else {
                std::fill(n->sens.begin(), n->sens.end(), T(0));
            }
        }
        for (size_t i = nodes.size(); i-- > 0;) nodes[i]->backward(*this);
    }
};

template <class T> struct PosNode : Node<T> {
    void forward(Engine<T>&, bool) override {}
};

// Distance3D: |x1-x2| (src/coord_basic.cpp:13-66)
template <class T> struct DistNode : Node<T> {
    vector<int> a1, a2;
    vector<V3<T>> der;
    DistNode(const H5& h) {
        auto id = h.ri("id");
        int n = int(id.size() / 2);
        for (int i = 0; i < n; ++i) { a1.push_back(id[2 * i]); a2.push_back(id[2 * i + 1]); }
        this->alloc(n, 1);
        der.resize(size_t(n));
    }
    void forward(Engine<T>& e, bool) override {
        auto& p1 = e.arg(*this, 0); auto& p2 = e.arg(*this, 1);
        for (int i = 0; i < this->n_elem; ++i) {
            V3<T> d = ld3(&p1.out[3 * size_t(a1[i])]) - ld3(&p2.out[3 * size_t(a2[i])]);
            T r = std::sqrt(mag2(d));
            this->out[size_t(i)] = r;
            der[size_t(i)] = r != T(0) ? d * (T(1) / r) : V3<T>();
        }
    }
    void backward(Engine<T>& e) override {
        auto& p1 = e.arg(*this, 0); auto& p2 = e.arg(*this, 1);
        for (int i = 0; i < this->n_elem; ++i) {
            T s = this->sens[size_t(i)];
            add3(&p1.sens[3 * size_t(a1[i])], der[size_t(i)] * s);
            add3(&p2.sens[3 * size_t(a2[i])], der[size_t(i)] * (-s));
        }
    }
};

// Angle: cosine of the angle at atom 3 (src/coord_basic.cpp:183-243)
template <class T> struct AngleNode : Node<T> {
    vector<int> id;
    vector<V3<T>> d1, d2;
    AngleNode(const H5& h) {
        id = h.ri("id");
        int n = int(id.size() / 3);
        this->alloc(n, 1);
        d1.resize(size_t(n)); d2.resize(size_t(n));
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            V3<T> a = ld3(&p.out[3 * size_t(id[3 * i])]), b = ld3(&p.out[3 * size_t(id[3 * i + 1])]),
                  c = ld3(&p.out[3 * size_t(id[3 * i + 2])]);
            V3<T> x1 = a - c, x2 = b - c;
            T i1 = T(1) / std::sqrt(mag2(x1)), i2 = T(1) / std::sqrt(mag2(x2));
            V3<T> h1 = x1 * i1, h2 = x2 * i2;
            T dp = dot(h1, h2);
            this->out[size_t(i)] = dp;
            d1[size_t(i)] = (h2 - h1 * dp) * i1;
            d2[size_t(i)] = (h1 - h2 * dp) * i2;
        }
    }
    void backward(Engine<T>& e) override {
        auto& p = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            T s = this->sens[size_t(i)];
            add3(&p.sens[3 * size_t(id[3 * i])], d1[size_t(i)] * s);
            add3(&p.sens[3 * size_t(id[3 * i + 1])], d2[size_t(i)] * s);
            add3(&p.sens[3 * size_t(id[3 * i + 2])], (d1[size_t(i)] + d2[size_t(i)]) * (-s));
        }
    }
};

// Dihedral angle, -80 deg for missing terminal atoms (src/coord_basic.cpp:311-374,
// src/vector_math.h:766-800)
template <class T> struct DihedralNode : Node<T> {
    vector<int> id;
    vector<V3<T>> jac;
    DihedralNode(const H5& h) {
        id = h.ri("id");
        int n = int(id.size() / 4);
        this->alloc(n, 1);
        jac.resize(size_t(4 * n));
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            const int* a = &id[4 * size_t(i)];
            if (a[0] < 0 || a[3] < 0) { this->out[size_t(i)] = T(-1.3963f); continue; }
            V3<T> r1 = ld3(&p.out[3 * size_t(a[0])]), r2 = ld3(&p.out[3 * size_t(a[1])]),
                  r3 = ld3(&p.out[3 * size_t(a[2])]), r4 = ld3(&p.out[3 * size_t(a[3])]);
            V3<T> F = r1 - r2, G = r2 - r3, H = r4 - r3;
            V3<T> A = cross(F, G), B = cross(H, G), C = cross(B, A);
            T iA = T(1) / mag2(A), iB = T(1) / mag2(B);
            T G2 = mag2(G), iG = T(1) / std::sqrt(G2), Gm = G2 * iG;
            V3<T> dd1 = A * (-Gm * iA), dd4 = B * (Gm * iB);
            V3<T> fm = A * (dot(F, G) * iA * iG) - B * (dot(H, G) * iB * iG);
            jac[4 * size_t(i) + 0] = dd1;
            jac[4 * size_t(i) + 1] = fm - dd1;
            jac[4 * size_t(i) + 2] = -dd4 - fm;
            jac[4 * size_t(i) + 3] = dd4;
            this->out[size_t(i)] = std::atan2(dot(C, G), dot(A, B) * Gm);
        }
    }
    void backward(Engine<T>& e) override {
        auto& p = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            const int* a = &id[4 * size_t(i)];
            if (a[0] < 0 || a[3] < 0) continue;
            T s = this->sens[size_t(i)];
            for (int k = 0; k < 4; ++k) add3(&p.sens[3 * size_t(a[k])], jac[4 * size_t(i) + k] * s);
        }
    }
};

// Spring on one component of a coordinate, optional periodic wrap (src/spring.cpp:9-81)
template <class T> struct SpringNode : Node<T> {
    vector<int> id;
    vector<T> eq, k;
    int dim1;
    bool pbc;
    T box;
    SpringNode(const H5& h) {
        this->potential_node = true;
        id = h.ri("id");
        eq = h.rf<T>("equil_dist");
        k = h.rf<T>("spring_const");
        dim1 = int(h.attr("dim1"));
        pbc = h.attr("pbc") != 0;
        box = T(h.attr("box_len"));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& c = e.arg(*this, 0);
        this->pot = 0;
        for (size_t i = 0; i < id.size(); ++i) {
            T x = c.out[size_t(id[i]) * c.width + dim1];
            T ex = x - eq[i], s2 = ex * ex;
            if (ex == T(0)) continue;
            if (pbc) {
                T e1 = x - eq[i] - box, e2 = x - eq[i] + box;
                if (e1 * e1 < s2) { s2 = e1 * e1; ex = e1; }
                if (e2 * e2 < s2) { s2 = e2 * e2; ex = e2; }
            }
            if (energy) this->pot += T(0.5) * k[i] * s2;
            c.sens[size_t(id[i]) * c.width + dim1] += k[i] * ex;
        }
    }
};

// rama_coord: paste (phi, psi) rows (PasteRama, src/coord_map.cpp:69-110)
template <class T> struct PasteRamaNode : Node<T> {
    vector<int> i1, i2;
    PasteRamaNode(const H5& h) {
        i1 = h.ri("index_pos1");
        i2 = h.ri("index_pos2");
        this->alloc(int(i1.size()), 2);
    }
    void forward(Engine<T>& e, bool) override {
        auto& a = e.arg(*this, 0); auto& b = e.arg(*this, 1);
        for (int i = 0; i < this->n_elem; ++i) {
            this->out[2 * size_t(i)] = a.out[size_t(i1[size_t(i)]) * a.width];
            this->out[2 * size_t(i) + 1] = b.out[size_t(i2[size_t(i)]) * b.width];
        }
    }
    void backward(Engine<T>& e) override {
        auto& a = e.arg(*this, 0); auto& b = e.arg(*this, 1);
        for (int i = 0; i < this->n_elem; ++i) {
            a.sens[size_t(i1[size_t(i)]) * a.width] += this->sens[2 * size_t(i)];
            b.sens[size_t(i2[size_t(i)]) * b.width] += this->sens[2 * size_t(i) + 1];
        }
    }
};

// cat_pos: concatenation of two coordinate nodes (src/coord_map.cpp:112-161)
template <class T> struct CatPosNode : Node<T> {
    vector<int> i1, i2;
    CatPosNode(const H5& h) {
        i1 = h.ri("index_pos1");
        i2 = h.ri("index_pos2");
        this->alloc(int(i1.size() + i2.size()), int(h.attr("n_dim")));
    }
    void forward(Engine<T>& e, bool) override {
        auto& a = e.arg(*this, 0); auto& b = e.arg(*this, 1);
        int w = this->width;
        for (size_t i = 0; i < i1.size(); ++i)
            for (int d = 0; d < w; ++d) this->out[i * w + d] = a.out[size_t(i1[i]) * a.width + d];
        for (size_t i = 0; i < i2.size(); ++i)
            for (int d = 0; d < w; ++d) this->out[(i + i1.size()) * w + d] = b.out[size_t(i2[i]) * b.width + d];
    }
    void backward(Engine<T>& e) override {
        auto& a = e.arg(*this, 0); auto& b = e.arg(*this, 1);
        int w = this->width;
        for (size_t i = 0; i < i1.size(); ++i)
            for (int d = 0; d < w; ++d) a.sens[size_t(i1[i]) * a.width + d] += this->sens[i * w + d];
        for (size_t i = 0; i < i2.size(); ++i)
            for (int d = 0; d < w; ++d) b.sens[size_t(i2[i]) * b.width + d] += this->sens[(i + i1.size()) * w + d];
    }
};

// Rama map potential: periodic bicubic per residue (src/rama_map_pot.cpp:15-94)
template <class T> struct RamaMapNode : Node<T> {
    vector<int> res, map_id;
    Periodic2D<T> sp;
    RamaMapNode(const H5& h) {
        this->potential_node = true;
        res = h.ri("residue_id");
        map_id = h.ri("rama_map_id");
        auto d = h.dims("rama_pot");
        if (d.size() != 3 || d[1] != d[2]) throw Err("rama_pot must be (n_layer, n, n)");
        sp.fit(int(d[0]), int(d[1]), int(d[2]), h.rd("rama_pot"));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& r = e.arg(*this, 0);
        const T scale = T(sp.nx) * (T(0.5f / float(M_PI)) - T(1e-7f));
        const T shift = T(float(M_PI));
        this->pot = 0;
        for (size_t i = 0; i < res.size(); ++i) {
            T* ro = &r.out[size_t(res[i]) * 2];
            T v, dx, dy;
            sp.eval(map_id[i], (ro[0] + shift) * scale, (ro[1] + shift) * scale, v, dx, dy);
            if (energy) this->pot += v;
            r.sens[size_t(res[i]) * 2] += dx * scale;
            r.sens[size_t(res[i]) * 2 + 1] += dy * scale;
        }
    }
};

// RamaMap2: Rama map potential scaled per residue by a switch coordinate
// lambda (row = position in the residue list) (src/rama_map_pot.cpp:96-175)
template <class T> struct RamaMap2Node : Node<T> {
    vector<int> res, map_id;
    Periodic2D<T> sp;
    RamaMap2Node(const H5& h) {
        this->potential_node = true;
        res = h.ri("residue_id");
        map_id = h.ri("rama_map_id");
        auto d = h.dims("rama_pot");
        if (d.size() != 3 || d[1] != d[2]) throw Err("rama_pot must be (n_layer, n, n)");
        sp.fit(int(d[0]), int(d[1]), int(d[2]), h.rd("rama_pot"));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& r = e.arg(*this, 0);
        auto& lam = e.arg(*this, 1);
        const T scale = T(sp.nx) * (T(0.5f / float(M_PI)) - T(1e-7f));
        const T shift = T(float(M_PI));
        this->pot = 0;
        for (size_t i = 0; i < res.size(); ++i) {
            T* ro = &r.out[size_t(res[i]) * 2];
            T v, dx, dy;
            sp.eval(map_id[i], (ro[0] + shift) * scale, (ro[1] + shift) * scale, v, dx, dy);
            T l = lam.out[i * size_t(lam.width)];
            if (energy) this->pot += v * l;
            r.sens[size_t(res[i]) * 2] += dx * scale * l;
            r.sens[size_t(res[i]) * 2 + 1] += dy * scale * l;
            lam.sens[i * size_t(lam.width)] += v;
        }
    }
};

// SigmoidCoord: compact sigmoid of one column of a coordinate, or its
// complement for a negative sign (src/coord_map.cpp:609-675)
template <class T> struct SigmoidCoordNode : Node<T> {
    vector<int> id;
    vector<T> c, s, sign, der;
    int dim1;
    SigmoidCoordNode(const H5& h) {
        id = h.ri("id");
        c = h.rf<T>("c");
        s = h.rf<T>("s");
        sign = h.rf<T>("sign");
        dim1 = int(h.attr("dim1"));
        this->alloc(int(id.size()), 1);
        der.assign(id.size(), T(0));
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0);
        for (size_t i = 0; i < id.size(); ++i) {
            T v, d;
            compact_sigmoid(p.out[size_t(id[i]) * p.width + dim1] - c[i], s[i], v, d);
            this->out[i] = sign[i] > T(0) ? v : T(1) - v;
            der[i] = sign[i] > T(0) ? d : -d;
        }
    }
    void backward(Engine<T>& e) override {
        auto& p = e.arg(*this, 0);
        for (size_t i = 0; i < id.size(); ++i) p.sens[size_t(id[i]) * p.width + dim1] += this->sens[i] * der[i];
    }
};

// Add, Mean and Multiply of two coordinates into n_size rows of n_dim
// (src/coord_operator.cpp:15-112, 114-226, 228-351).  As in the reference,
// Multiply scales the sensitivity passed to each factor by that factor's own
// last value written to the row, not by the other factor.
template <class T> struct CombineNode : Node<T> {
    enum Op { ADD, MEAN, MUL } op;
    vector<int> ip1, ip2, o1, o2, d1, d2, count;
    vector<T> s1, s2, scl;
    CombineNode(const H5& h, Op o) : op(o) {
        int n_size = int(h.attr("n_size")), n_dim = int(h.attr("n_dim"));
        this->alloc(n_size, n_dim);
        ip1 = h.ri("id_pos1"); ip2 = h.ri("id_pos2");
        o1 = h.ri("id1_out"); o2 = h.ri("id2_out");
        d1 = h.ri("dim1"); d2 = h.ri("dim2");
        if (int(d1.size()) != n_dim || int(d2.size()) != n_dim || o1.size() != ip1.size() || o2.size() != ip2.size())
            throw Err("inconsistent sizes");
        count.assign(size_t(n_size), 0);
        for (int i : o1) { if (i < 0 || i >= n_size) throw Err("output id out of range"); ++count[size_t(i)]; }
        for (int i : o2) { if (i < 0 || i >= n_size) throw Err("output id out of range"); ++count[size_t(i)]; }
        s1.assign(size_t(n_size), T(1));
        s2.assign(size_t(n_size), T(1));
        scl.assign(size_t(n_size), T(1));
        if (op == MEAN)
            for (int i = 0; i < n_size; ++i) scl[size_t(i)] = count[size_t(i)] ? T(1) / T(count[size_t(i)]) : T(1);
    }
    void forward(Engine<T>& e, bool) override {
        auto& a = e.arg(*this, 0); auto& b = e.arg(*this, 1);
        int nd = this->width;
        std::fill(this->out.begin(), this->out.end(), op == MUL ? T(1) : T(0));
        auto pass = [&](const vector<int>& ip, const vector<int>& oo, const vector<int>& dd, Node<T>& src,
                        vector<T>& keep) {
            for (size_t i = 0; i < ip.size(); ++i)
                for (int d = 0; d < nd; ++d) {
                    T v = src.out[size_t(ip[i]) * src.width + dd[size_t(d)]];
                    T& o = this->out[size_t(oo[i]) * nd + d];
                    if (op == MUL) { o *= v; keep[size_t(oo[i])] = v; }
                    else o += v * scl[size_t(oo[i])];
                }
        };
        pass(ip1, o1, d1, a, s2);
        pass(ip2, o2, d2, b, s1);
        if (op == MUL)
            for (int i = 0; i < this->n_elem; ++i)
                if (!count[size_t(i)])
                    for (int d = 0; d < nd; ++d) this->out[size_t(i) * nd + d] = T(0);
    }
    void backward(Engine<T>& e) override {
        auto& a = e.arg(*this, 0); auto& b = e.arg(*this, 1);
        int nd = this->width;
        auto pass = [&](const vector<int>& ip, const vector<int>& oo, const vector<int>& dd, Node<T>& dst,
                        const vector<T>& f) {
            for (size_t i = 0; i < ip.size(); ++i)
                for (int d = 0; d < nd; ++d)
                    dst.sens[size_t(ip[i]) * dst.width + dd[size_t(d)]] +=
                        this->sens[size_t(oo[i]) * nd + d] * f[size_t(oo[i])];
        };
        pass(ip1, o1, d1, a, op == MUL ? s2 : scl);
        pass(ip2, o2, d2, b, op == MUL ? s1 : scl);
    }
};

// Sum: one row of n_dim, the weighted sum of chosen rows of the argument.
// As in the reference, the adjoint weights entry i by weight[id_pos[i]]
// rather than weight[i] (src/coord_operator.cpp:353-406); an id_pos outside
// the weight list is refused instead of read past its end.
template <class T> struct SumNode : Node<T> {
    vector<int> ip, dim;
    vector<T> wt;
    SumNode(const H5& h) {
        ip = h.ri("id_pos");
        dim = h.ri("dim");
        wt = h.rf<T>("weight");
        int nd = int(h.attr("n_dim"));
        if (int(dim.size()) != nd || wt.size() != ip.size()) throw Err("inconsistent sizes");
        for (int i : ip)
            if (i < 0 || i >= int(wt.size())) throw Err("id_pos outside the weight list");
        this->alloc(1, nd);
    }
    void forward(Engine<T>& e, bool) override {
        auto& a = e.arg(*this, 0);
        for (int d = 0; d < this->width; ++d) {
            T acc = 0;
            for (size_t i = 0; i < ip.size(); ++i) acc += wt[i] * a.out[size_t(ip[i]) * a.width + dim[size_t(d)]];
            this->out[size_t(d)] = acc;
        }
    }
    void backward(Engine<T>& e) override {
        auto& a = e.arg(*this, 0);
        for (size_t i = 0; i < ip.size(); ++i)
            for (int d = 0; d < this->width; ++d)
                a.sens[size_t(ip[i]) * a.width + dim[size_t(d)]] += this->sens[size_t(d)] * wt[size_t(ip[i])];
    }
};

// SigmoidEnergy / SigmoidLEnergy: a + b * compact_sigmoid(x - c, s) on one
// column, optionally times a switch coordinate lambda; with use_cutoff only
// x in [min, max] counts, otherwise x beyond c -+ 1/s takes the plateau
// value (src/sigmoid_energy.cpp:9-91, 93-185)
template <class T> struct SigmoidEnergyNode : Node<T> {
    bool with_lambda;
    vector<int> id, id2;
    vector<T> a, b, c, s, lo, hi;
    int dim1;
    bool use_cutoff;
    SigmoidEnergyNode(const H5& h, bool lam) : with_lambda(lam) {
        this->potential_node = true;
        id = h.ri(lam ? "id1" : "id");
        if (lam) id2 = h.ri("id2");
        a = h.rf<T>("a"); b = h.rf<T>("b"); c = h.rf<T>("c"); s = h.rf<T>("s");
        lo = h.rf<T>("min"); hi = h.rf<T>("max");
        dim1 = int(h.attr("dim1"));
        use_cutoff = h.attr("use_cutoff") != 0;
        if (!use_cutoff)
            for (size_t i = 0; i < id.size(); ++i) {
                lo[i] = c[i] - T(1) / s[i];
                hi[i] = c[i] + T(1) / s[i];
            }
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& p = e.arg(*this, 0);
        this->pot = 0;
        for (size_t i = 0; i < id.size(); ++i) {
            T x = p.out[size_t(id[i]) * p.width + dim1];
            T l = with_lambda ? e.arg(*this, 1).out[size_t(id2[i]) * e.arg(*this, 1).width] : T(1);
            if (use_cutoff && (x > hi[i] || x < lo[i])) continue;
            if (x > hi[i]) {
                if (energy) this->pot += l * a[i];
            } else if (x < lo[i]) {
                if (energy) this->pot += l * (a[i] + b[i]);
            } else {
                T v, d;
                compact_sigmoid(x - c[i], s[i], v, d);
                if (energy) this->pot += l * (a[i] + b[i] * v);
                p.sens[size_t(id[i]) * p.width + dim1] += l * b[i] * d;
                if (with_lambda) e.arg(*this, 1).sens[size_t(id2[i]) * e.arg(*this, 1).width] += a[i] + b[i] * v;
            }
        }
    }
};

// Const1D/2D/3D: fixed rows of k values, or chosen components of chosen rows
// of the argument taken at the first evaluation and kept
// (ConstantCoord1D/2D/3D, src/coord_const.cpp:9-179); one row per entry of id
template <class T> struct ConstNode : Node<T> {
    bool by_coord, done = false;
    vector<int> id;
    int dim[3] = {0, 0, 0};
    ConstNode(const H5& h, int k) {
        by_coord = h.attr("initialized_by_coord") != 0;
        if (k == 1) dim[0] = int(h.attr("dim"));
        else
            for (int c = 0; c < k; ++c) dim[c] = int(h.attr(c == 0 ? "dim1" : (c == 1 ? "dim2" : "dim3")));
        id = h.ri("id");
        this->alloc(int(id.size()), k);
        if (!by_coord) {
            auto v = h.rd("value");
            if (v.size() != id.size() * size_t(k)) throw Err("value must hold k numbers per entry of id");
            for (size_t i = 0; i < v.size(); ++i) this->out[i] = T(float(v[i]));
        }
    }
    void forward(Engine<T>& e, bool) override {
        if (!by_coord || done) return;
        auto& p = e.arg(*this, 0);
        int k = this->width;
        for (size_t i = 0; i < id.size(); ++i)
            for (int c = 0; c < k; ++c) this->out[size_t(k) * i + size_t(c)] = p.out[size_t(id[i]) * p.width + dim[c]];
        done = true;
    }
};

// depth coordinate of a point for the membrane terms: z, or on a curved
// bilayer sign * (|x - centre| - radius), with its gradient
template <class T> T membrane_depth(const T* x, const T* cc, bool curved, T sign, T radius, T grad[3]) {
    if (!curved) {
        grad[0] = grad[1] = 0;
        grad[2] = 1;
        return x[2];
    }
    V3<T> d = V3<T>(x[0], x[1], x[2]) - V3<T>(cc[0], cc[1], cc[2]);
    T dist = std::sqrt(mag2(d)), r = T(1) / dist;
    // the reference's gradient uses (x, y, z - sign*radius*-1), which is
    // x - centre for the centre (0, 0, -sign*radius) the config writes
    grad[0] = sign * x[0] * r;
    grad[1] = sign * x[1] * r;
    grad[2] = sign * (x[2] - sign * radius * T(-1)) * r;
    return sign * (dist - radius);
}

// left/right mirrored clamped spline of depth: ll * f(z) + lr * f(-z), with
// ll the compact sigmoid switch at left_right_node; returns value, d/dz
template <class T> void mirrored_spline(const T* c, int n, T z, T z0, T zs, T lr_node, T lr_sharp, T& v, T& dv) {
    T sl, dsl;
    compact_sigmoid(z - lr_node, lr_sharp, sl, dsl);
    T ll = sl, lr = T(1) - sl, dll = dsl, dlr = -dsl;
    T fl, dfl, fr, dfr;
    clamped(c, (z - z0) * zs, n, fl, dfl);
    clamped(c, (-z - z0) * zs, n, fr, dfr);
    v = ll * fl + lr * fr;
    dv = ll * dfl * zs + dll * fl - lr * dfr * zs + dlr * fr;
}

// CB membrane energy: burial level (weighted environment coverage) blended
// over burial bins by compact sigmoids, times the mirrored depth spline of
// the residue type and bin (MembraneCBPotential, src/membrane_potential.cpp:221-486)
template <class T> struct MembraneCBNode : Node<T> {
    vector<int> cb_index, res_type;
    vector<T> weights, bl_nodes, coeff;
    int n_restype, n_bl, n_node;
    T bl_sharp, lr_node, lr_sharp, radius, sign, z0, zs;
    bool curved;
    MembraneCBNode(const H5& h) {
        this->potential_node = true;
        cb_index = h.ri("cb_index");
        res_type = h.ri("res_type");
        weights = h.rf<T>("weights");
        bl_nodes = h.rf<T>("bl_nodes");
        auto d = h.dims("coeff");
        if (d.size() != 3) throw Err("coeff must be (n_restype, n_bl, n_node)");
        n_restype = int(d[0]); n_bl = int(d[1]); n_node = int(d[2]);
        if (int(bl_nodes.size()) != n_bl - 1) throw Err("bl_nodes must have n_bl - 1 entries");
        coeff = h.rf<T>("coeff");
        bl_sharp = T(float(h.attr("bl_range_sharpness")));
        lr_node = T(float(h.attr("left_right_node")));
        lr_sharp = T(float(h.attr("left_right_sharpness")));
        curved = h.attr("use_curvature") != 0;
        radius = T(float(h.attr("curvature_radius")));
        sign = T(float(h.attr("curvature_sign")));
        z0 = T(float(h.attr("z_start")));
        zs = T(float(h.attr("z_scale")));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& cb = e.arg(*this, 0);
        auto& env = e.arg(*this, 1);
        auto& cc = e.arg(*this, 2);
        radius = cc.out[2] * T(-1) * sign;
        T pot = 0;
        const size_t nb = static_cast<size_t>(n_bl);
        vector<T> s1(nb), ds1(nb), s2(nb), ds2(nb), bs(nb), dbs(nb);
        for (size_t nr = 0; nr < cb_index.size(); ++nr) {
            int rt = res_type[nr], ri = cb_index[nr];
            T bl = 0;
            for (int a = 0; a < n_restype; ++a) bl += weights[size_t(a)] * env.out[size_t(ri) * n_restype + a];
            for (int i = 0; i < n_bl - 1; ++i) {
                T v, dd;
                compact_sigmoid(bl - bl_nodes[size_t(i)], bl_sharp, v, dd);
                s1[size_t(i)] = v; ds1[size_t(i)] = dd;
                compact_sigmoid(bl_nodes[size_t(i)] - bl, bl_sharp, v, dd);
                s2[size_t(i)] = v; ds2[size_t(i)] = -dd;
            }
            bs[0] = s1[0]; dbs[0] = ds1[0];
            bs[size_t(n_bl - 1)] = s2[size_t(n_bl - 2)]; dbs[size_t(n_bl - 1)] = ds2[size_t(n_bl - 2)];
            for (int i = 0; i < n_bl - 2; ++i) {
                bs[size_t(i + 1)] = s2[size_t(i)] * s1[size_t(i + 1)];
                dbs[size_t(i + 1)] = ds2[size_t(i)] * s1[size_t(i + 1)] + s2[size_t(i)] * ds1[size_t(i + 1)];
            }
            T* x = &cb.out[size_t(ri) * cb.width];
            T gz[3];
            T z = membrane_depth(x, &cc.out[0], curved, sign, radius, gz);
            T dz = 0, dbl = 0;
            for (int i = 0; i < n_bl; ++i) {
                T f, df;
                mirrored_spline(&coeff[(size_t(rt) * n_bl + size_t(i)) * n_node], n_node, z, z0, zs, lr_node, lr_sharp,
                                f, df);
                pot += bs[size_t(i)] * f;
                dbl += dbs[size_t(i)] * f;
                dz += bs[size_t(i)] * df;
            }
            T* xs = &cb.sens[size_t(ri) * cb.width];
            for (int k = 0; k < 3; ++k) xs[k] += dz * gz[k];
            for (int a = 0; a < n_restype; ++a) env.sens[size_t(ri) * n_restype + a] += weights[size_t(a)] * dbl;
        }
        this->pot = energy ? pot : T(0);
    }
};

// backbone H/O membrane energy: (1 - p)^2 f0(depth) + (1 - (1 - p)^2) f1(depth)
// with p the hbond probability of the donor/acceptor (column 6 of
// protein_hbond) (MembraneHBPotential, src/membrane_potential.cpp:488-672)
template <class T> struct MembraneHBNode : Node<T> {
    vector<int> hb_index, hb_type;
    vector<T> coeff;
    int n_node;
    T lr_node, lr_sharp, radius, sign, z0, zs;
    bool curved;
    MembraneHBNode(const H5& h) {
        this->potential_node = true;
        hb_index = h.ri("hb_index");
        hb_type = h.ri("hb_type");
        auto d = h.dims("coeff");
        if (d.size() != 3 || d[0] != 2 || d[1] != 2) throw Err("coeff must be (2, 2, n_node)");
        n_node = int(d[2]);
        coeff = h.rf<T>("coeff");
        lr_node = T(float(h.attr("left_right_node")));
        lr_sharp = T(float(h.attr("left_right_sharpness")));
        curved = h.attr("use_curvature") != 0;
        radius = T(float(h.attr("curvature_radius")));
        sign = T(float(h.attr("curvature_sign")));
        z0 = T(float(h.attr("z_start")));
        zs = T(float(h.attr("z_scale")));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& hb = e.arg(*this, 0);
        auto& cc = e.arg(*this, 1);
        radius = cc.out[2] * T(-1) * sign;
        T pot = 0;
        for (size_t nv = 0; nv < hb_index.size(); ++nv) {
            int rt = hb_type[nv], ri = hb_index[nv];
            T* x = &hb.out[size_t(ri) * hb.width];
            T* xs = &hb.sens[size_t(ri) * hb.width];
            T gz[3];
            T z = membrane_depth(x, &cc.out[0], curved, sign, radius, gz);
            T p = x[6], u = T(1) - p;
            T f1, df1, f2, df2;
            mirrored_spline(&coeff[size_t(rt) * 2 * n_node], n_node, z, z0, zs, lr_node, lr_sharp, f1, df1);
            mirrored_spline(&coeff[(size_t(rt) * 2 + 1) * n_node], n_node, z, z0, zs, lr_node, lr_sharp, f2, df2);
            T w1 = u * u, w2 = T(1) - u * u;
            pot += w1 * f1 + w2 * f2;
            xs[6] += -T(2) * u * f1 + T(2) * u * f2;
            for (int k = 0; k < 3; ++k) xs[k] += (w1 * df1 + w2 * df2) * gz[k];
        }
        this->pot = energy ? pot : T(0);
    }
};

// ---------------------------------------------------------------- surface --
// Lipid-exposed residues of a membrane protein (Surface, src/surface.cpp:54-696).
// Residues whose N, CA, C and CB all lie inside the slab |z| < half +
// zbuffer are the TM residues.  For each of n_rotation turns about z (by
// a * pi/2 / n_rotation about the TM CBs' xy centre) the atoms and their
// auxiliary points (a circle of the atom radius in the yz and xz planes)
// are put on a voxel grid; the outermost occupied voxels of each x- and
// y-row (method 0), or those next to lipid voxels found by a layer-wise
// flood fill from the grid border (method 1), are surface voxels; within
// them a grid of n_smallgrid cells per voxel picks the outermost CB per
// fine row, and each picked CB gets a share of a lateral force proportional
// to the surface area.  Output per residue: the fraction of turns since the
// residue was first picked, and the mean picked force (x, y) turned back.
// The node is a discrete function of float roundings, so it runs in float
// whatever T is, in the reference's order of operations.  Its state carries
// over between evaluations as the reference's does: the TM list beyond the
// current TM count and the forces of residues not in the slab keep the
// values of earlier evaluations.  The node has no derivative
// (src/surface.cpp:692-694).
namespace surface_arith {
// The steps whose rounding decides voxel membership, each rounded
// separately in the reference's order of operations (the library is built
// without contraction into fused multiply-adds).  Against the reference
// engine on 138 random frames the surface fractions matched exactly and the
// force columns to a few units in the last place, except for 3 frames where
// one turn picked a different CB for a fine row; fused forms of the turns,
// the auxiliary offsets and the grid origin, a centre summed in partial sums
// and reciprocal products in place of the divisions changed none of that.
inline float rot_x(float rx, float c, float s, float dx, float dy) {
    float a = c * dx, b = rx + a, e = s * dy;
    return b - e;
}
inline float rot_y(float ry, float c, float s, float dx, float dy) {
    float a = s * dx, b = ry + a, e = c * dy;
    return b + e;
}
inline float aux_add(float x, float a, float r) {
    float d = a * r;
    return x + d;
}
}  // namespace surface_arith

struct SurfaceCore {
    int method = 1, n_rot = 0, n_aux = 0, ngz = 0, snx = 1, sny = 1, snz = 1, n_res = 0;
    float half = 0, zbuf = 0, radius = 0, tm_min = 0, tm_max = 0, gx = 0, gy = 0, gz = 0, r_gz = 0, r_nrot = 0;
    vector<int> index_cb, used, tm_list;
    vector<float> aux, sfx, sfy, cp, sp, cm, sm;
    struct Vox {
        int nx, ny, nz;
        vector<int> v;
        int& at(int i, int j, int k) {
            if (i < 0 || j < 0 || k < 0 || i >= nx || j >= ny || k >= nz) throw Err("surface voxel out of the grid");
            return v[(size_t(i) * ny + j) * nz + k];
        }
    };
    void init(const H5& h) {
        method = int(h.attr("method_type"));
        if (method != 0 && method != 1) throw Err("surface method_type must be 0 or 1");
        index_cb = h.ri("index_cb");
        n_res = int(index_cb.size());
        n_rot = int(h.attr("n_rotation"));
        if (n_rot < 1) throw Err("surface needs n_rotation >= 1");
        auto ad = h.dims("auxiliary_point");
        if (ad.size() != 2 || ad[1] != 2) throw Err("auxiliary_point must be (n_aux, 2)");
        n_aux = int(ad[0]);
        aux = h.rf<float>("auxiliary_point");
        r_nrot = float(1. / n_rot);
        float dangle = float(0.5 * double(3.141592653589793f) * double(r_nrot));
        half = float(h.attr("half_thickness"));
        zbuf = float(h.attr("zbuffer"));
        radius = float(h.attr("atom_radius"));
        tm_min = -half - zbuf;
        tm_max = half + zbuf;
        ngz = int(h.attr("n_gridz"));
        if (ngz < 2) throw Err("surface needs n_gridz >= 2");
        gx = float(h.attr("len_gridx"));
        gy = float(h.attr("len_gridy"));
        float ext = tm_max - tm_min;
        ext = ext + 2 * radius;
        gz = float((double(ext) + 0.1) / ngz);
        r_gz = 1.f / gz;
        snx = int(h.attr("n_smallgridx"));
        sny = int(h.attr("n_smallgridy"));
        snz = int(h.attr("n_smallgridz"));
        if (snx < 1 || sny < 1 || snz < 1) throw Err("surface small grids need >= 1 cell");
        int excl = int(h.attr("exclusion"));
        if (excl == 1) used = h.ri("included_list");
        else {
            used.resize(size_t(n_res));
            for (int i = 0; i < n_res; ++i) used[size_t(i)] = i;
        }
        for (int r : used)
            if (r < 0 || r >= n_res) throw Err("surface included_list entry out of range");
        tm_list.assign(used.size(), 0);
        sfx.assign(size_t(n_res), 0.f);
        sfy.assign(size_t(n_res), 0.f);
        step = dangle;
    }
    float step = 0.f;
    void angles() {
        cp.clear(); sp.clear(); cm.clear(); sm.clear();
        for (int a = 0; a < n_rot; ++a) {
            float ang = float(a) * step;
            cp.push_back(std::cos(ang));
            sp.push_back(std::sin(ang));
            cm.push_back(std::cos(-ang));
            sm.push_back(std::sin(-ang));
        }
    }
    static void rotate(vector<float>& x, vector<float>& y, float rx, float ry, float c, float s, int n) {
        for (int i = 0; i < n; ++i) {
            float dx = x[size_t(i)] - rx, dy = y[size_t(i)] - ry;
            if (dx == 0 && dy == 0) continue;
            x[size_t(i)] = surface_arith::rot_x(rx, c, s, dx, dy);
            y[size_t(i)] = surface_arith::rot_y(ry, c, s, dx, dy);
        }
    }
    static void minmax(const vector<float>& x, int n, bool init, float& mn, float& mx) {
        for (int i = 0; i < n; ++i) {
            float v = x[size_t(i)];
            if (!init) { mn = mx = v; init = true; }
            else if (v > mx) mx = v;
            else if (v < mn) mn = v;
        }
    }
    // pos(atom, d): float coordinate d of row `atom` of the concatenated
    // backbone + CB positions; out: n_res x 3
    template <class P> void compute(P pos, float* out) {
        using surface_arith::aux_add;
        angles();
        int n_tm = 0;
        for (int nr : used) {
            auto in = [&](int row) { float z = pos(row, 2); return z < tm_max && z > tm_min; };
            if (in(nr * 3) && in(nr * 3 + 1) && in(nr * 3 + 2) && in(index_cb[size_t(nr)])) tm_list[size_t(n_tm++)] = nr;
        }
        vector<int> tc(static_cast<size_t>(n_res), 0), surf_cb(static_cast<size_t>(n_tm), 0);
        const size_t nt = static_cast<size_t>(n_tm);
        vector<float> bbx(3 * nt), bby(3 * nt), bbz(3 * nt), cbx(nt), cby(nt), cbz(nt), fx(nt), fy(nt);
        for (int ii = 0; ii < n_tm; ++ii) {
            int nr = tm_list[size_t(ii)];
            for (int j = 0; j < 3; ++j) {
                bbx[size_t(ii * 3 + j)] = pos(nr * 3 + j, 0);
                bby[size_t(ii * 3 + j)] = pos(nr * 3 + j, 1);
                bbz[size_t(ii * 3 + j)] = pos(nr * 3 + j, 2);
            }
            cbx[size_t(ii)] = pos(index_cb[size_t(nr)], 0);
            cby[size_t(ii)] = pos(index_cb[size_t(nr)], 1);
            cbz[size_t(ii)] = pos(index_cb[size_t(nr)], 2);
            sfx[size_t(nr)] = 0.f;
            sfy[size_t(nr)] = 0.f;
        }
        float cx = 0.f, cy = 0.f;
        for (int i = 0; i < n_tm; ++i) { cx += cbx[size_t(i)]; cy += cby[size_t(i)]; }
        cx /= float(n_tm);
        cy /= float(n_tm);
        for (int a = 0; a < n_rot; ++a) {
            rotate(cbx, cby, cx, cy, cp[size_t(a)], sp[size_t(a)], n_tm);
            // only the first n_tm backbone entries turn (src/surface.cpp:240)
            rotate(bbx, bby, cx, cy, cp[size_t(a)], sp[size_t(a)], n_tm);
            float minx = 0.f, maxx = 0.f, miny = 0.f, maxy = 0.f;
            minmax(bbx, 3 * n_tm, false, minx, maxx);
            minmax(cbx, n_tm, true, minx, maxx);
            minmax(bby, 3 * n_tm, false, miny, maxy);
            minmax(cby, n_tm, true, miny, maxy);
            minx -= radius; maxx += radius; miny -= radius; maxy += radius;
            float lenx = maxx - minx, leny = maxy - miny;
            int ngx = int((double(lenx) + 0.1) / double(gx)) + 3;
            int ngy = int((double(leny) + 0.1) / double(gy)) + 3;
            int ngz_ = ngz;
            float blx = float(ngx) * gx, bly = float(ngy) * gy;
            float side[3], s1[3], s2[3];
            float hx = 0.5f * (blx - lenx), hy = 0.5f * (bly - leny);
            side[0] = minx - hx;
            side[1] = miny - hy;
            side[2] = tm_min - radius;
            s1[0] = float(ngx) / blx; s1[1] = float(ngy) / bly; s1[2] = r_gz;
            s2[0] = float(snx * ngx) / blx; s2[1] = float(sny * ngy) / bly; s2[2] = float(snz) * r_gz;
            auto cell = [&](float x, float y, float z, const float* sc, int v[3]) {
                float p[3] = {x, y, z};
                for (int d = 0; d < 3; ++d) {
                    float t = p[d] - side[d];
                    v[d] = int(std::floor(t * sc[d]));
                }
            };
            Vox V{ngx, ngy, ngz_, vector<int>(size_t(ngx) * ngy * ngz_, -1)};
            vector<int> vid(size_t(4 * n_tm) * 3);
            auto mark_atom = [&](float x, float y, float z, int iv) {
                int v[3];
                cell(x, y, z, s1, v);
                for (int d = 0; d < 3; ++d) vid[size_t(iv) * 3 + d] = v[d];
                V.at(v[0], v[1], v[2]) = 1;
                for (int j = 0; j < n_aux; ++j) {
                    float ax = aux[size_t(2 * j)], az = aux[size_t(2 * j + 1)];
                    cell(x + 0.0f, aux_add(y, ax, radius), aux_add(z, az, radius), s1, v);
                    V.at(v[0], v[1], v[2]) = 1;
                }
                for (int j = 0; j < n_aux; ++j) {
                    float ax = aux[size_t(2 * j)], az = aux[size_t(2 * j + 1)];
                    cell(aux_add(x, ax, radius), y + 0.0f, aux_add(z, az, radius), s1, v);
                    V.at(v[0], v[1], v[2]) = 1;
                }
            };
            for (int nr = 0; nr < n_tm; ++nr) {
                for (int i = 0; i < 3; ++i)
                    mark_atom(bbx[size_t(nr * 3 + i)], bby[size_t(nr * 3 + i)], bbz[size_t(nr * 3 + i)], nr * 4 + i);
                mark_atom(cbx[size_t(nr)], cby[size_t(nr)], cbz[size_t(nr)], nr * 4 + 3);
            }
            int nxz = ngx * ngz_, nyz = ngy * ngz_;
            if (method == 0) {
                int big = ngx * ngy * ngz_;
                vector<int> xmn(size_t(nyz), big), xmx(size_t(nyz), -1), ymn(size_t(nxz), big), ymx(size_t(nxz), -1);
                for (int i = 0; i < ngx; ++i)
                    for (int j = 0; j < ngy; ++j)
                        for (int k = 0; k < ngz_; ++k)
                            if (V.at(i, j, k) == 1) {
                                int ik = i * ngz_ + k, jk = j * ngz_ + k;
                                xmn[size_t(jk)] = std::min(xmn[size_t(jk)], i);
                                xmx[size_t(jk)] = std::max(xmx[size_t(jk)], i);
                                ymn[size_t(ik)] = std::min(ymn[size_t(ik)], j);
                                ymx[size_t(ik)] = std::max(ymx[size_t(ik)], j);
                            }
                for (int jk = 0; jk < nyz; ++jk) {
                    int j = jk / ngz_, k = jk % ngz_;
                    if (xmn[size_t(jk)] < big) V.at(xmn[size_t(jk)], j, k) += 10;
                    if (xmx[size_t(jk)] > -1) V.at(xmx[size_t(jk)], j, k) += 100;
                }
                for (int ik = 0; ik < nxz; ++ik) {
                    int i = ik / ngz_, k = ik % ngz_;
                    if (ymn[size_t(ik)] < big) V.at(i, ymn[size_t(ik)], k) += 1000;
                    if (ymx[size_t(ik)] > -1) V.at(i, ymx[size_t(ik)], k) += 10000;
                }
            } else {
                for (int k = 0; k < ngz_; ++k) {
                    for (int i = 0; i < ngx; ++i) { V.at(i, 0, k) = 0; V.at(i, ngy - 1, k) = 0; }
                    for (int j = 0; j < ngy; ++j) { V.at(0, j, k) = 0; V.at(ngx - 1, j, k) = 0; }
                }
                // empty voxels next (3 x 3 in the layer) to a lipid voxel become
                // lipid until none changes; the tail layers also want the
                // neighbour's voxel in the layer towards the head group lipid.
                // The result is the closure, whatever the order of visits.
                auto fill = [&](int k, int kref) {
                    bool changed = true;
                    while (changed) {
                        changed = false;
                        for (int i = 1; i < ngx - 1; ++i)
                            for (int j = 1; j < ngy - 1; ++j) {
                                if (V.at(i, j, k) != -1) continue;
                                bool hit = false;
                                for (int ii = i - 1; ii < i + 2 && !hit; ++ii)
                                    for (int jj = j - 1; jj < j + 2 && !hit; ++jj)
                                        hit = V.at(ii, jj, k) == 0 && (kref < 0 || V.at(ii, jj, kref) == 0);
                                if (hit) { V.at(i, j, k) = 0; changed = true; }
                            }
                    }
                };
                fill(0, -1);
                fill(ngz_ - 1, -1);
                for (int k = 1; k < ngz_ / 2; ++k) fill(k, k - 1);
                // the top layer was closed above; the reference's second pass
                // over it (reading one layer past the grid) converts nothing
                for (int k = ngz_ - 2; k >= ngz_ / 2; --k) fill(k, k + 1);
                for (int i = 1; i < ngx - 1; ++i)
                    for (int j = 1; j < ngy - 1; ++j)
                        for (int k = 0; k < ngz_; ++k)
                            if (V.at(i, j, k) > 0) {
                                int add = 0;
                                if (V.at(i - 1, j, k) == 0) add += 10;
                                if (V.at(i + 1, j, k) == 0) add += 100;
                                if (V.at(i, j - 1, k) == 0) add += 1000;
                                if (V.at(i, j + 1, k) == 0) add += 10000;
                                V.at(i, j, k) += add;
                            }
            }
            int big = ngx * snx + ngy * sny + ngz_ * snz;
            int zs = ngz_ * snz;
            size_t nfx = size_t(sny * snz) * size_t(nyz), nfy = size_t(snx * snz) * size_t(nxz);
            vector<int> fxmn(nfx, big), fxmx(nfx, -1), fymn(nfy, big), fymx(nfy, -1);
            vector<int> ixmn(nfx, -1), ixmx(nfx, -1), iymn(nfy, -1), iymx(nfy, -1);
            auto at_fx = [&](vector<int>& a, int idx) -> int& {
                if (idx < 0 || size_t(idx) >= a.size()) throw Err("surface fine row out of the grid");
                return a[size_t(idx)];
            };
            auto labels = [&](int iv, int& v2, int& v3, int& v4, int& v5) {
                int t = V.at(vid[size_t(iv) * 3], vid[size_t(iv) * 3 + 1], vid[size_t(iv) * 3 + 2]);
                v5 = t / 10000;
                v4 = (t % 10000) / 1000;
                v3 = ((t % 10000) % 1000) / 100;
                v2 = (((t % 10000) % 1000) % 100) / 10;
                return t;
            };
            // surface backbone atoms and the auxiliary points of surface
            // backbone atoms and CBs widen the fine extremes
            auto widen = [&](float x, float y, float z, int iv, bool self) {
                int v2, v3, v4, v5;
                if (labels(iv, v2, v3, v4, v5) <= 1) return;
                int q[3];
                cell(x, y, z, s2, q);
                if (self) {
                    int kj = q[1] * zs + q[2], ki = q[0] * zs + q[2];
                    if (v2 == 1 && q[0] < at_fx(fxmn, kj)) fxmn[size_t(kj)] = q[0];
                    if (v3 == 1 && q[0] > at_fx(fxmx, kj)) fxmx[size_t(kj)] = q[0];
                    if (v4 == 1 && q[1] < at_fx(fymn, ki)) fymn[size_t(ki)] = q[1];
                    if (v5 == 1 && q[1] > at_fx(fymx, ki)) fymx[size_t(ki)] = q[1];
                }
                for (int j = 0; j < n_aux; ++j) {
                    float ax = aux[size_t(2 * j)], az = aux[size_t(2 * j + 1)];
                    int a[3];
                    cell(x + 0.0f, aux_add(y, ax, radius), aux_add(z, az, radius), s2, a);
                    int kj = a[1] * zs + q[2];
                    if (v2 == 1 && a[0] < at_fx(fxmn, kj)) fxmn[size_t(kj)] = a[0];
                    if (v3 == 1 && a[0] > at_fx(fxmx, kj)) fxmx[size_t(kj)] = a[0];
                }
                for (int j = 0; j < n_aux; ++j) {
                    float ax = aux[size_t(2 * j)], az = aux[size_t(2 * j + 1)];
                    int a[3];
                    cell(aux_add(x, ax, radius), y + 0.0f, aux_add(z, az, radius), s2, a);
                    int ki = a[0] * zs + q[2];
                    if (v4 == 1 && a[1] < at_fx(fymn, ki)) fymn[size_t(ki)] = a[1];
                    if (v5 == 1 && a[1] > at_fx(fymx, ki)) fymx[size_t(ki)] = a[1];
                }
            };
            for (int nr = 0; nr < n_tm; ++nr)
                for (int i = 0; i < 3; ++i)
                    widen(bbx[size_t(nr * 3 + i)], bby[size_t(nr * 3 + i)], bbz[size_t(nr * 3 + i)], nr * 4 + i, true);
            for (int nr = 0; nr < n_tm; ++nr) widen(cbx[size_t(nr)], cby[size_t(nr)], cbz[size_t(nr)], nr * 4 + 3, false);
            // the outermost surface CB of each fine row (the last in residue
            // order on ties)
            for (int nr = 0; nr < n_tm; ++nr) {
                int v2, v3, v4, v5;
                if (labels(nr * 4 + 3, v2, v3, v4, v5) <= 1) continue;
                int q[3];
                cell(cbx[size_t(nr)], cby[size_t(nr)], cbz[size_t(nr)], s2, q);
                int kj = q[1] * zs + q[2], ki = q[0] * zs + q[2];
                if (v2 == 1 && q[0] <= at_fx(fxmn, kj)) { fxmn[size_t(kj)] = q[0]; ixmn[size_t(kj)] = nr; }
                if (v3 == 1 && q[0] >= at_fx(fxmx, kj)) { fxmx[size_t(kj)] = q[0]; ixmx[size_t(kj)] = nr; }
                if (v4 == 1 && q[1] <= at_fx(fymn, ki)) { fymn[size_t(ki)] = q[1]; iymn[size_t(ki)] = nr; }
                if (v5 == 1 && q[1] >= at_fx(fymx, ki)) { fymx[size_t(ki)] = q[1]; iymx[size_t(ki)] = nr; }
            }
            int n_xmn = 0, n_xmx = 0, n_ymn = 0, n_ymx = 0, c_xmn = 0, c_xmx = 0, c_ymn = 0, c_ymx = 0;
            for (int v : fxmn) n_xmn += v < big;
            for (int v : fxmx) n_xmx += v > -1;
            for (int v : fymn) n_ymn += v < big;
            for (int v : fymx) n_ymx += v > -1;
            for (int v : ixmn) c_xmn += v > -1;
            for (int v : ixmx) c_xmx += v > -1;
            for (int v : iymn) c_ymn += v > -1;
            for (int v : iymx) c_ymx += v > -1;
            float area_xz = gx / float(snx) * gz / float(snz);
            float area_yz = gy / float(sny) * gz / float(snz);
            float a_xmn = float(n_xmn) * area_yz, a_xmx = float(n_xmx) * area_yz;
            float a_ymn = float(n_ymn) * area_xz, a_ymx = float(n_ymx) * area_xz;
            float ax_ = a_xmn > a_xmx ? a_xmn : a_xmx;
            float ay_ = a_ymn > a_ymx ? a_ymn : a_ymx;
            float tfx = float(double(ax_) * 2.428602e-5), tfy = float(double(ay_) * 2.428602e-5);
            float f_xmn = tfx / float(c_xmn), f_xmx = tfx / float(c_xmx);
            float f_ymn = tfy / float(c_ymn), f_ymx = tfy / float(c_ymx);
            std::fill(fx.begin(), fx.end(), 0.f);
            std::fill(fy.begin(), fy.end(), 0.f);
            for (int nr : ixmn) if (nr >= 0) { surf_cb[size_t(nr)] = 1; fx[size_t(nr)] = f_xmn; }
            for (int nr : ixmx) if (nr >= 0) { surf_cb[size_t(nr)] = 1; fx[size_t(nr)] -= f_xmx; }
            for (int nr : iymn) if (nr >= 0) { surf_cb[size_t(nr)] = 1; fy[size_t(nr)] = f_ymn; }
            for (int nr : iymx) if (nr >= 0) { surf_cb[size_t(nr)] = 1; fy[size_t(nr)] -= f_ymx; }
            for (int ns = 0; ns < n_tm; ++ns)
                if (surf_cb[size_t(ns)]) tc[size_t(tm_list[size_t(ns)])] += 1;
            for (int i = 0; i < n_tm; ++i) {
                float f0 = fx[size_t(i)], f1 = fy[size_t(i)];
                if (f0 == 0 && f1 == 0) continue;
                fx[size_t(i)] = surface_arith::rot_x(0.f, cm[size_t(a)], sm[size_t(a)], f0, f1);
                fy[size_t(i)] = surface_arith::rot_y(0.f, cm[size_t(a)], sm[size_t(a)], f0, f1);
            }
            rotate(cbx, cby, cx, cy, cm[size_t(a)], sm[size_t(a)], n_tm);
            rotate(bbx, bby, cx, cy, cm[size_t(a)], sm[size_t(a)], n_tm);
            for (int ns = 0; ns < n_tm; ++ns) {
                if (!surf_cb[size_t(ns)]) continue;
                int nr = tm_list[size_t(ns)];
                sfx[size_t(nr)] += fx[size_t(ns)];
                sfy[size_t(nr)] += fy[size_t(ns)];
            }
        }
        // every entry of the TM list, including those left from earlier
        // evaluations beyond the current count (src/surface.cpp:675-679)
        for (int nr : tm_list) {
            if (tc[size_t(nr)] <= 0) continue;
            sfx[size_t(nr)] /= float(tc[size_t(nr)]);
            sfy[size_t(nr)] /= float(tc[size_t(nr)]);
        }
        for (int nr = 0; nr < n_res; ++nr) {
            out[3 * nr] = tc[size_t(nr)] > 0 ? float(tc[size_t(nr)]) * r_nrot : 0.f;
            out[3 * nr + 1] = sfx[size_t(nr)];
            out[3 * nr + 2] = sfy[size_t(nr)];
        }
    }
};

template <class T> struct SurfaceNode : Node<T> {
    SurfaceCore S;
    SurfaceNode(const H5& h) {
        S.init(h);
        this->alloc(S.n_res, 3);
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0);
        if (p.width < 3) throw Err("surface needs coordinates of width 3");
        for (int i = 0; i < S.n_res; ++i)
            if (S.index_cb[size_t(i)] < 0 || S.index_cb[size_t(i)] >= p.n_elem || 3 * i + 2 >= p.n_elem)
                throw Err("surface index_cb out of range");
        vector<float> out(size_t(S.n_res) * 3);
        S.compute([&](int row, int d) { return float(p.out[size_t(row) * p.width + d]); }, out.data());
        for (size_t i = 0; i < out.size(); ++i) this->out[i] = T(out[i]);
    }
};

// CB membrane energy with the surface score (MembraneSurfCBPotential,
// src/membrane_potential.cpp:674-983): as cb_membrane_potential, but inside
// the slab every burial bin but the first weights its depth spline by the
// residue's surface score s and adds the residue type's inner spline with
// weight 1 - s (outside the slab, bins past the first use s = 1)
template <class T> struct MembraneSurfCBNode : Node<T> {
    vector<int> cb_index, res_type;
    vector<T> weights, bl_nodes, coeff, coeff_inner;
    int n_restype, n_bl, n_node;
    T bl_sharp, lr_node, lr_sharp, radius, sign, z0, zs, half;
    bool curved;
    MembraneSurfCBNode(const H5& h) {
        this->potential_node = true;
        cb_index = h.ri("cb_index");
        res_type = h.ri("res_type");
        weights = h.rf<T>("weights");
        bl_nodes = h.rf<T>("bl_nodes");
        auto d = h.dims("coeff");
        if (d.size() != 3) throw Err("coeff must be (n_restype, n_bl, n_node)");
        n_restype = int(d[0]); n_bl = int(d[1]); n_node = int(d[2]);
        auto di = h.dims("coeff_inner");
        if (di.size() != 2 || int(di[0]) != n_restype || int(di[1]) != n_node)
            throw Err("coeff_inner must be (n_restype, n_node)");
        if (int(bl_nodes.size()) != n_bl - 1) throw Err("bl_nodes must have n_bl - 1 entries");
        if (res_type.size() != cb_index.size()) throw Err("res_type needs one entry per cb_index");
        coeff = h.rf<T>("coeff");
        coeff_inner = h.rf<T>("coeff_inner");
        bl_sharp = T(float(h.attr("bl_range_sharpness")));
        lr_node = T(float(h.attr("left_right_node")));
        lr_sharp = T(float(h.attr("left_right_sharpness")));
        curved = h.attr("use_curvature") != 0;
        radius = T(float(h.attr("curvature_radius")));
        sign = T(float(h.attr("curvature_sign")));
        z0 = T(float(h.attr("z_start")));
        zs = T(float(h.attr("z_scale")));
        half = T(float(h.attr("half_thickness")));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& cb = e.arg(*this, 0);
        auto& env = e.arg(*this, 1);
        auto& sf = e.arg(*this, 2);
        auto& cc = e.arg(*this, 3);
        radius = cc.out[2] * T(-1) * sign;
        T pot = 0;
        const size_t nb = static_cast<size_t>(n_bl);
        vector<T> s1(nb), ds1(nb), s2(nb), ds2(nb), bs(nb), dbs(nb);
        for (size_t nr = 0; nr < cb_index.size(); ++nr) {
            int rt = res_type[nr], ri = cb_index[nr];
            T bl = 0;
            for (int a = 0; a < n_restype; ++a) bl += weights[size_t(a)] * env.out[size_t(ri) * n_restype + a];
            for (int i = 0; i < n_bl - 1; ++i) {
                T v, dd;
                compact_sigmoid(bl - bl_nodes[size_t(i)], bl_sharp, v, dd);
                s1[size_t(i)] = v; ds1[size_t(i)] = dd;
                compact_sigmoid(bl_nodes[size_t(i)] - bl, bl_sharp, v, dd);
                s2[size_t(i)] = v; ds2[size_t(i)] = -dd;
            }
            bs[0] = s1[0]; dbs[0] = ds1[0];
            bs[nb - 1] = s2[nb - 2]; dbs[nb - 1] = ds2[nb - 2];
            for (int i = 0; i < n_bl - 2; ++i) {
                bs[size_t(i + 1)] = s2[size_t(i)] * s1[size_t(i + 1)];
                dbs[size_t(i + 1)] = ds2[size_t(i)] * s1[size_t(i + 1)] + s2[size_t(i)] * ds1[size_t(i + 1)];
            }
            T* x = &cb.out[size_t(ri) * cb.width];
            T gz[3];
            T z = membrane_depth(x, &cc.out[0], curved, sign, radius, gz);
            T sl, dsl;
            compact_sigmoid(z - lr_node, lr_sharp, sl, dsl);
            T ll = sl, lr = T(1) - sl, dll = dsl, dlr = -dsl;
            T cl = (z - z0) * zs, cr = (-z - z0) * zs;
            T dz = 0, dbl = 0;
            for (int i = 0; i < n_bl; ++i) {
                T sv = (i > 0 && (z > half || z < -half)) ? T(1) : sf.out[size_t(ri) * sf.width];
                const T* c = &coeff[(size_t(rt) * n_bl + size_t(i)) * n_node];
                T v, dv;
                clamped(c, cl, n_node, v, dv);
                T fl = v * sv, dfl = dv * zs * sv;
                clamped(c, cr, n_node, v, dv);
                T fr = v * sv, dfr = -dv * sv * zs;
                if (sv < T(1)) {
                    const T* ci = &coeff_inner[size_t(rt) * n_node];
                    clamped(ci, cl, n_node, v, dv);
                    fl += v * (T(1) - sv);
                    dfl += dv * (T(1) - sv) * zs;
                    clamped(ci, cr, n_node, v, dv);
                    fr += v * (T(1) - sv);
                    dfr -= dv * (T(1) - sv) * zs;
                }
                T fs = ll * fl + lr * fr;
                T dfs = ll * dfl + dll * fl + lr * dfr + dlr * fr;
                pot += bs[size_t(i)] * fs;
                dbl += dbs[size_t(i)] * fs;
                dz += bs[size_t(i)] * dfs;
            }
            T* xs = &cb.sens[size_t(ri) * cb.width];
            for (int k = 0; k < 3; ++k) xs[k] += dz * gz[k];
            for (int a = 0; a < n_restype; ++a) env.sens[size_t(ri) * n_restype + a] += weights[size_t(a)] * dbl;
        }
        this->pot = energy ? pot : T(0);
    }
};

// backbone H/O membrane energy with the surface score
// (MembraneSurfHBPotential, src/membrane_potential.cpp:989-1259): the
// bonded / free splines of hb_membrane_potential weighted by
// outer = s * compact_sigmoid(burial - 2.5, 2) of the residue, plus the
// inner tables weighted by 1 - outer (s = 1 outside the slab)
template <class T> struct MembraneSurfHBNode : Node<T> {
    vector<int> hb_index, hb_type, hb_res;
    vector<T> weights, coeff, coeff_inner;
    int n_node, n_restype;
    T lr_node, lr_sharp, radius, sign, z0, zs, half;
    bool curved;
    MembraneSurfHBNode(const H5& h) {
        this->potential_node = true;
        hb_index = h.ri("hb_index");
        hb_type = h.ri("hb_type");
        hb_res = h.ri("hb_res");
        if (hb_type.size() != hb_index.size() || hb_res.size() != hb_index.size())
            throw Err("hb_type and hb_res need one entry per hb_index");
        weights = h.rf<T>("weights");
        n_restype = int(weights.size());
        auto d = h.dims("coeff");
        if (d.size() != 3 || d[0] != 2 || d[1] != 2) throw Err("coeff must be (2, 2, n_node)");
        n_node = int(d[2]);
        auto di = h.dims("coeff_inner");
        if (di.size() != 3 || di[0] != 2 || di[1] != 2 || int(di[2]) != n_node)
            throw Err("coeff_inner must be (2, 2, n_node)");
        coeff = h.rf<T>("coeff");
        coeff_inner = h.rf<T>("coeff_inner");
        lr_node = T(float(h.attr("left_right_node")));
        lr_sharp = T(float(h.attr("left_right_sharpness")));
        curved = h.attr("use_curvature") != 0;
        radius = T(float(h.attr("curvature_radius")));
        sign = T(float(h.attr("curvature_sign")));
        z0 = T(float(h.attr("z_start")));
        zs = T(float(h.attr("z_scale")));
        half = T(float(h.attr("half_thickness")));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& hb = e.arg(*this, 0);
        auto& env = e.arg(*this, 1);
        auto& sf = e.arg(*this, 2);
        auto& cc = e.arg(*this, 3);
        radius = cc.out[2] * T(-1) * sign;
        T pot = 0;
        for (size_t nv = 0; nv < hb_index.size(); ++nv) {
            int rt = hb_type[nv], ri = hb_index[nv], rr = hb_res[nv];
            T* x = &hb.out[size_t(ri) * hb.width];
            T* xs = &hb.sens[size_t(ri) * hb.width];
            T gz[3];
            T z = membrane_depth(x, &cc.out[0], curved, sign, radius, gz);
            T bl = 0;
            for (int a = 0; a < n_restype; ++a) bl += weights[size_t(a)] * env.out[size_t(rr) * n_restype + a];
            T sb, dsb;
            compact_sigmoid(bl - T(2.5), T(2), sb, dsb);
            T sv = sf.out[size_t(rr) * sf.width];
            if (z > half || z < -half) sv = T(1);
            T outer = sv * sb, d_outer = sv * dsb, inner = T(1) - outer, d_inner = -d_outer;
            T p = x[6], u = T(1) - p, w1 = u * u, w2 = T(1) - w1;
            T f1, df1, f2, df2, dZ = 0, dHB = 0, dBL = 0;
            if (outer > T(0)) {
                mirrored_spline(&coeff[size_t(rt) * 2 * n_node], n_node, z, z0, zs, lr_node, lr_sharp, f1, df1);
                mirrored_spline(&coeff[(size_t(rt) * 2 + 1) * n_node], n_node, z, z0, zs, lr_node, lr_sharp, f2, df2);
                pot += w1 * outer * f1 + w2 * outer * f2;
                dHB += -T(2) * u * outer * f1 + T(2) * u * outer * f2;
                dBL += w1 * d_outer * f1 + w2 * d_outer * f2;
                dZ += w1 * outer * df1 + w2 * outer * df2;
            }
            if (inner > T(0)) {
                mirrored_spline(&coeff_inner[size_t(rt) * 2 * n_node], n_node, z, z0, zs, lr_node, lr_sharp, f1, df1);
                mirrored_spline(&coeff_inner[(size_t(rt) * 2 + 1) * n_node], n_node, z, z0, zs, lr_node, lr_sharp, f2,
                                df2);
                pot += w1 * inner * f1 + w2 * inner * f2;
                dHB += -T(2) * u * inner * f1 + T(2) * u * inner * f2;
                dBL += w1 * d_inner * f1 + w2 * d_inner * f2;
                dZ += w1 * inner * df1 + w2 * inner * df2;
            }
            for (int k = 0; k < 3; ++k) xs[k] += dZ * gz[k];
            xs[6] += dHB;
            for (int a = 0; a < n_restype; ++a) env.sens[size_t(rr) * n_restype + a] += weights[size_t(a)] * dBL;
        }
        this->pot = energy ? pot : T(0);
    }
};

// lateral pressure on surface residues (MembraneLateralPotential,
// src/membrane_potential.cpp:1262-1354): a force (no energy) of
// s * p(z) * compact_sigmoid(burial - midpoint, sharpness) along the
// residue's surface force direction (columns 1-2 of the surface node), with
// p the clamped spline of the pressure profile over z.  The reference
// indexes the per-residue burial and type arrays by the residue number, so
// every cb_index entry must be below the number of entries.
template <class T> struct LateralNode : Node<T> {
    vector<int> cb_index, restype;
    vector<T> weights, midpoint, sharpness, params;
    T min_z, inv_dz, half;
    int n_knot;
    LateralNode(const H5& h) {
        this->potential_node = true;
        cb_index = h.ri("cb_index");
        restype = h.ri("restypes");
        weights = h.rf<T>("weights");
        midpoint = h.rf<T>("cov_midpoint");
        sharpness = h.rf<T>("cov_sharpness");
        params = h.rf<T>("params");
        min_z = T(float(h.attr("min_z")));
        inv_dz = T(float(h.attr("inv_dz")));
        half = T(float(h.attr("half_thickness")));
        n_knot = int(h.attr("n_knot"));
        int n = int(cb_index.size());
        if (int(restype.size()) != n) throw Err("restypes needs one entry per cb_index");
        if (weights.size() != 20 || midpoint.size() != 20 || sharpness.size() != 20)
            throw Err("weights, cov_midpoint and cov_sharpness need 20 entries");
        if (int(params.size()) != n_knot) throw Err("params needs n_knot entries");
        for (int r : cb_index)
            if (r < 0 || r >= n) throw Err("cb_index entries must be below the number of entries");
        for (int t : restype)
            if (t < 0 || t >= 20) throw Err("restypes out of range");
    }
    void forward(Engine<T>& e, bool) override {
        auto& cb = e.arg(*this, 0);
        auto& env = e.arg(*this, 1);
        auto& sf = e.arg(*this, 2);
        int n = int(cb_index.size());
        vector<T> wbl(size_t(n), T(0));
        for (int r = 0; r < n; ++r)
            for (int a = 0; a < 20; ++a) wbl[size_t(r)] += weights[size_t(a)] * env.out[size_t(r) * 20 + a];
        for (int i = 0; i < n; ++i) {
            int r = cb_index[size_t(i)];
            T z = cb.out[size_t(r) * cb.width + 2];
            T sv = sf.out[size_t(r) * sf.width];
            if (z > half || z < -half) sv = T(1);
            int t = restype[size_t(r)];
            T cs, dcs;
            compact_sigmoid(wbl[size_t(r)] - midpoint[size_t(t)], sharpness[size_t(t)], cs, dcs);
            if (sv <= T(0) || cs == T(0)) continue;
            T v, dv;
            clamped(params.data(), (z - min_z) * inv_dz, n_knot, v, dv);
            T fm = sv * v;
            cb.sens[size_t(r) * cb.width] -= fm * cs * sf.out[size_t(r) * sf.width + 1];
            cb.sens[size_t(r) * cb.width + 1] -= fm * cs * sf.out[size_t(r) * sf.width + 2];
        }
        this->pot = T(0);
    }
};

// Rigid frame per residue from N, CA, C (AffineAlignment, src/eig.cpp:277-470).
// Output (center, quaternion); sensitivity slots 3..5 carry the torque.
template <class T> struct AffineNode : Node<T> {
    vector<int> atoms;
    vector<T> ref;  // (n,3,3)
    vector<T> evals, evecs;
    AffineNode(const H5& h) {
        atoms = h.ri("atoms");
        ref = h.rf<T>("ref_geom");
        int n = int(atoms.size() / 3);
        this->alloc(n, 7);
        evals.resize(size_t(4 * n));
        evecs.resize(size_t(16 * n));
    }
    static void dF_dR(int i, int j, T dF[4][4]) {
        // F as a linear function of R (key matrix of the quaternion fit)
        for (int a = 0; a < 4; ++a)
            for (int b = 0; b < 4; ++b) dF[a][b] = 0;
        auto set = [&](int a, int b, T v) { dF[a][b] += v; if (a != b) dF[b][a] += v; };
        if (i == 0 && j == 0) { set(0, 0, 1); set(1, 1, 1); set(2, 2, -1); set(3, 3, -1); }
        if (i == 1 && j == 1) { set(0, 0, 1); set(1, 1, -1); set(2, 2, 1); set(3, 3, -1); }
        if (i == 2 && j == 2) { set(0, 0, 1); set(1, 1, -1); set(2, 2, -1); set(3, 3, 1); }
        if (i == 1 && j == 2) { set(0, 1, 1); set(2, 3, 1); }
        if (i == 2 && j == 1) { set(0, 1, -1); set(2, 3, 1); }
        if (i == 2 && j == 0) { set(0, 2, 1); set(1, 3, 1); }
        if (i == 0 && j == 2) { set(0, 2, -1); set(1, 3, 1); }
        if (i == 0 && j == 1) { set(0, 3, 1); set(1, 2, 1); }
        if (i == 1 && j == 0) { set(0, 3, -1); set(1, 2, 1); }
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0);
        T Fg[4][4][4];
        for (int r = 0; r < this->n_elem; ++r) {
            V3<T> x[3];
            for (int a = 0; a < 3; ++a) x[a] = ld3(&p.out[3 * size_t(atoms[3 * size_t(r) + a])]);
            V3<T> c = (x[0] + x[1] + x[2]) * (T(1) / T(3));
            for (int a = 0; a < 3; ++a) x[a] -= c;
            T R[3][3];
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) {
                    R[i][j] = 0;
                    for (int a = 0; a < 3; ++a) R[i][j] += x[a][j] * ref[(size_t(r) * 3 + a) * 3 + i];
                }
            T F[4][4];
            F[0][0] = R[0][0] + R[1][1] + R[2][2];
            F[0][1] = R[1][2] - R[2][1];
            F[0][2] = R[2][0] - R[0][2];
            F[0][3] = R[0][1] - R[1][0];
            F[1][1] = R[0][0] - R[1][1] - R[2][2];
            F[1][2] = R[0][1] + R[1][0];
            F[1][3] = R[0][2] + R[2][0];
            F[2][2] = -R[0][0] + R[1][1] - R[2][2];
            F[2][3] = R[1][2] + R[2][1];
            F[3][3] = -R[0][0] - R[1][1] + R[2][2];
            for (int a = 0; a < 4; ++a)
                for (int b = 0; b < a; ++b) F[a][b] = F[b][a];
            // residues 4g..4g+3 are solved together, as the reference's SIMD groups are
            std::memcpy(Fg[r & 3], F, sizeof F);
            T* o = &this->out[7 * size_t(r)];
            o[0] = c.x; o[1] = c.y; o[2] = c.z;
            if ((r & 3) == 3 || r == this->n_elem - 1) {
                int r0 = r & ~3;
                qr4_group(r - r0 + 1, Fg, &evals[4 * size_t(r0)], &evecs[16 * size_t(r0)]);
                for (int l = r0; l <= r; ++l)
                    for (int k = 0; k < 4; ++k) this->out[7 * size_t(l) + 3 + k] = evecs[16 * size_t(l) + k];
            }
        }
    }
    void backward(Engine<T>& e) override {
        auto& p = e.arg(*this, 0);
        for (int r = 0; r < this->n_elem; ++r) {
            const T* s = &this->sens[7 * size_t(r)];
            const T* ev = &evecs[16 * size_t(r)];
            const T* q = ev;
            V3<T> tq(s[3], s[4], s[5]);
            // torque -> gradient along the quaternion tangent (src/eig.cpp:406-410)
            T qs[4] = {T(2) * (-tq.x * q[1] - tq.y * q[2] - tq.z * q[3]),
                       T(2) * (tq.x * q[0] + tq.y * q[3] - tq.z * q[2]),
                       T(2) * (tq.y * q[0] + tq.z * q[1] - tq.x * q[3]),
                       T(2) * (tq.z * q[0] + tq.x * q[2] - tq.y * q[1])};
            T proj[4];
            for (int k = 1; k < 4; ++k) {
                proj[k] = 0;
                for (int i = 0; i < 4; ++i) proj[k] += qs[i] * ev[4 * k + i];
                proj[k] /= (evals[4 * size_t(r)] - evals[4 * size_t(r) + k]);
            }
            for (int a = 0; a < 3; ++a) {
                V3<T> g(s[0] / T(3), s[1] / T(3), s[2] / T(3));
                T gd[3] = {g.x, g.y, g.z};
                for (int j = 0; j < 3; ++j) {
                    // d/d atom_a[j]: R(i,j) changes by ref_a[i]
                    T dF[4][4], tot[4][4];
                    for (int u = 0; u < 4; ++u)
                        for (int v = 0; v < 4; ++v) tot[u][v] = 0;
                    for (int i = 0; i < 3; ++i) {
                        T w = ref[(size_t(r) * 3 + a) * 3 + i];
                        dF_dR(i, j, dF);
                        for (int u = 0; u < 4; ++u)
                            for (int v = 0; v < 4; ++v) tot[u][v] += w * dF[u][v];
                    }
                    for (int k = 1; k < 4; ++k) {
                        T vfq = 0;
                        for (int u = 0; u < 4; ++u)
                            for (int v = 0; v < 4; ++v) vfq += ev[4 * k + u] * tot[u][v] * q[v];
                        gd[j] += proj[k] * vfq;
                    }
                }
                add3(&p.sens[3 * size_t(atoms[3 * size_t(r) + a])], V3<T>(gd[0], gd[1], gd[2]));
            }
        }
    }
};

// Placement of rigid-body points / vectors / scalars (PlacementNode,
// src/placement.cpp:233-314, FixedPlacement :102-167, RamaPlacement :20-99).
// sig: string of 'P' (point), 'V' (vector), 'S' (scalar).
template <class T> struct PlacementNode : Node<T> {
    string sig;
    bool rama;  // placement data from a (phi,psi) spline
    vector<int> aff_res, layer, rama_res;
    vector<T> data;  // fixed: (n_layer, width)
    Periodic2D<T> sp;
    vector<T> rama_deriv;  // per element: d value / d(x,y) scaled grid coords
    PlacementNode(const H5& h, const string& sig_, bool rama_) : sig(sig_), rama(rama_) {
        aff_res = h.ri("affine_residue");
        layer = h.ri("layer_index");
        int w = 0;
        for (char c : sig) w += c == 'S' ? 1 : 3;
        this->alloc(int(aff_res.size()), w);
        if (rama) {
            if (w != 1) throw Err("only scalar rama placement supported");
            rama_res = h.ri("rama_residue");
            auto d = h.dims("placement_data");
            sp.fit(int(d[0]), int(d[1]), int(d[2]), h.rd("placement_data"));
            rama_deriv.resize(2 * aff_res.size());
        } else {
            data = h.rf<T>("placement_data");
            auto d = h.dims("placement_data");
            if (int(d[1]) != w) throw Err("placement_data width mismatch");
        }
    }
    void forward(Engine<T>& e, bool) override {
        auto& af = e.arg(*this, 0);
        int w = this->width;
        for (int i = 0; i < this->n_elem; ++i) {
            const T* a = &af.out[7 * size_t(aff_res[size_t(i)])];
            T U[9];
            quat_to_rot(a + 3, U);
            V3<T> t(a[0], a[1], a[2]);
            T* o = &this->out[size_t(i) * w];
            if (rama) {
                auto& r = e.arg(*this, 1);
                const T sx = T(sp.nx) * (T(0.5f / float(M_PI)) - T(1e-7f));
                const T sy = T(sp.ny) * (T(0.5f / float(M_PI)) - T(1e-7f));
                const T* rr = &r.out[2 * size_t(rama_res[size_t(i)])];
                T v, dx, dy;
                sp.eval(layer[size_t(i)], (rr[0] + T(float(M_PI))) * sx, (rr[1] + T(float(M_PI))) * sy, v, dx, dy);
                o[0] = v;
                rama_deriv[2 * size_t(i)] = dx;
                rama_deriv[2 * size_t(i) + 1] = dy;
                continue;
            }
            const T* v = &data[size_t(layer[size_t(i)]) * w];
            int off = 0;
            for (char c : sig) {
                if (c == 'S') { o[off] = v[off]; off += 1; continue; }
                V3<T> x = rot(U, ld3(v + off));
                if (c == 'P') x += t;
                st3(o + off, x);
                off += 3;
            }
        }
    }
    void backward(Engine<T>& e) override {
        auto& af = e.arg(*this, 0);
        int w = this->width;
        for (int i = 0; i < this->n_elem; ++i) {
            const T* s = &this->sens[size_t(i) * w];
            if (rama) {
                auto& r = e.arg(*this, 1);
                const T sx = T(sp.nx) * (T(0.5f / float(M_PI)) - T(1e-7f));
                const T sy = T(sp.ny) * (T(0.5f / float(M_PI)) - T(1e-7f));
                r.sens[2 * size_t(rama_res[size_t(i)])] += sx * s[0] * rama_deriv[2 * size_t(i)];
                r.sens[2 * size_t(rama_res[size_t(i)]) + 1] += sy * s[0] * rama_deriv[2 * size_t(i) + 1];
                continue;
            }
            const T* a = &af.out[7 * size_t(aff_res[size_t(i)])];
            V3<T> t(a[0], a[1], a[2]);
            const T* o = &this->out[size_t(i) * w];
            V3<T> com, torque;
            int off = 0;
            for (char c : sig) {
                if (c == 'S') { off += 1; continue; }
                V3<T> sv = ld3(s + off), xv = ld3(o + off);
                if (c == 'P') { com += sv; torque += cross(xv - t, sv); }
                else torque += cross(xv, sv);
                off += 3;
            }
            T* as = &af.sens[7 * size_t(aff_res[size_t(i)])];
            add3(as, com);
            add3(as + 3, torque);
        }
    }
};

// weighted_pos: (bead xyz, exp(-E_1body)) (src/environment.cpp:489-533)
template <class T> struct WeightedPosNode : Node<T> {
    vector<int> ip, iw;
    WeightedPosNode(const H5& h) {
        ip = h.ri("index_pos");
        iw = h.ri("index_weight");
        this->alloc(int(ip.size()), 4);
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0); auto& en = e.arg(*this, 1);
        for (int i = 0; i < this->n_elem; ++i) {
            for (int d = 0; d < 3; ++d) this->out[4 * size_t(i) + d] = p.out[size_t(ip[size_t(i)]) * p.width + d];
            this->out[4 * size_t(i) + 3] = std::exp(-en.out[size_t(iw[size_t(i)]) * en.width]);
        }
    }
    void backward(Engine<T>& e) override {
        auto& p = e.arg(*this, 0); auto& en = e.arg(*this, 1);
        for (int i = 0; i < this->n_elem; ++i) {
            for (int d = 0; d < 3; ++d) p.sens[size_t(ip[size_t(i)]) * p.width + d] += this->sens[4 * size_t(i) + d];
            en.sens[size_t(iw[size_t(i)]) * en.width] -= this->out[4 * size_t(i) + 3] * this->sens[4 * size_t(i) + 3];
        }
    }
};

// Virtual H and O positions and bond directions (Infer_H_O, src/hbond.cpp:20-127)
template <class T> struct InferHONode : Node<T> {
    vector<int> id;
    vector<T> bl;
    vector<T> cache;  // prev, next, disp unit vectors + inverse magnitudes
    InferHONode(const H5& h) {
        auto di = h.ri("donors/id"), ai = h.ri("acceptors/id");
        auto db = h.rf<T>("donors/bond_length"), ab = h.rf<T>("acceptors/bond_length");
        id = di;
        id.insert(id.end(), ai.begin(), ai.end());
        bl = db;
        bl.insert(bl.end(), ab.begin(), ab.end());
        this->alloc(int(bl.size()), 6);
        cache.resize(12 * bl.size());
    }
    void forward(Engine<T>& e, bool) override {
        auto& p = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            V3<T> pc = ld3(&p.out[3 * size_t(id[3 * size_t(i)])]), cc = ld3(&p.out[3 * size_t(id[3 * size_t(i) + 1])]),
                  nc = ld3(&p.out[3 * size_t(id[3 * size_t(i) + 2])]);
            V3<T> pv = pc - cc; T pi = T(1) / std::sqrt(mag2(pv)); pv = pv * pi;
            V3<T> nv = nc - cc; T ni = T(1) / std::sqrt(mag2(nv)); nv = nv * ni;
            V3<T> dv = pv + nv; T di = T(1) / std::sqrt(mag2(dv)); dv = dv * di;
            T* c = &cache[12 * size_t(i)];
            st3(c, pv); c[3] = pi; st3(c + 4, nv); c[7] = ni; st3(c + 8, dv); c[11] = di;
            T* o = &this->out[6 * size_t(i)];
            st3(o, cc + dv * (-bl[size_t(i)]));
            st3(o + 3, -dv);
        }
    }
    void backward(Engine<T>& e) override {
        auto& p = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            const T* s = &this->sens[6 * size_t(i)];
            const T* c = &cache[12 * size_t(i)];
            V3<T> sp = ld3(s), sd = ld3(s + 3);
            V3<T> sneg = sd + sp * bl[size_t(i)];  // sensitivity w.r.t. -disp unit vector
            V3<T> pv = ld3(c), nv = ld3(c + 4), dv = ld3(c + 8);
            V3<T> snd = (dv * dot(dv, sneg) - sneg) * c[11];  // w.r.t. non-unit disp
            V3<T> snp = (pv * dot(pv, snd) - snd) * (-c[3]);
            V3<T> snn = (nv * dot(nv, snd) - snd) * (-c[7]);
            add3(&p.sens[3 * size_t(id[3 * size_t(i)])], snp);
            add3(&p.sens[3 * size_t(id[3 * size_t(i) + 1])], sp - snp - snn);
            add3(&p.sens[3 * size_t(id[3 * size_t(i) + 2])], snn);
        }
    }
};

// ------------------------------------------------------ interaction graph --
// Pair list of an InteractionGraph in the reference's edge order
// (PairlistComputation, src/interaction_graph.h:51-258): candidate pairs are
// enumerated by (i1 block of 4, i2, i1 lane), filtered by dist2 < cutoff^2 and
// the id exclusion rule.
enum ExclRule { EX_ROTAMER, EX_SEQ1, EX_SEQ2 };

inline bool acceptable(ExclRule r, int a, int b) {
    switch (r) {
        case EX_ROTAMER: return (unsigned(a) >> 4) != (unsigned(b) >> 4);
        case EX_SEQ1: return (a - b > 1) || (b - a > 1);
        case EX_SEQ2: return (a - b > 2) || (b - a > 2);
    }
    return false;
}

template <class T> void find_pairs(bool symmetric, int n1, int n2, const vector<T>& x1, const vector<T>& x2,
                                   const vector<int>& id1, const vector<int>& id2, T cutoff, ExclRule rule,
                                   vector<std::pair<int, int>>& edges) {
    edges.clear();
    T c2 = cutoff * cutoff;
    for (int b = 0; b < n1; b += 4) {
        for (int i2 = symmetric ? b + 1 : 0; i2 < n2; ++i2) {
            for (int l = 0; l < 4; ++l) {
                int i1 = b + l;
                if (i1 >= n1) break;
                if (symmetric && !(i1 < i2)) continue;
                T dx = x1[3 * size_t(i1)] - x2[3 * size_t(i2)];
                T dy = x1[3 * size_t(i1) + 1] - x2[3 * size_t(i2) + 1];
                T dz = x1[3 * size_t(i1) + 2] - x2[3 * size_t(i2) + 2];
                T d2 = dx * dx + dy * dy + dz * dz;
                if (!(d2 < c2)) continue;
                if (!acceptable(rule, id1[size_t(i1)], id2[size_t(i2)])) continue;
                edges.emplace_back(i1, i2);
            }
        }
    }
}

// Quadspline bead-bead / backbone-bead coverage (quadspline, src/bead_interaction.h:31-85)
template <class T> T quadspline(int n_ka, int n_k, T inv_dtheta, T inv_dx, const T* p, const T* x1, const T* x2,
                                T* d1, T* d2) {
    V3<T> disp = ld3(x2) - ld3(x1), r1 = ld3(x1 + 3), r2 = ld3(x2 + 3);
    T dist2 = mag2(disp), inv_dist = T(1) / std::sqrt(dist2);
    T dc = dist2 * (inv_dist * inv_dx);
    V3<T> u = disp * inv_dist;
    T c1 = dot(r1, u), c2 = -dot(r2, u);
    T a1v, a1d, a2v, a2d, wv, wd, nv, nd;
    deboor(p, (c1 + T(1)) * inv_dtheta + T(1), a1v, a1d);
    deboor(p + n_ka, (c2 + T(1)) * inv_dtheta + T(1), a2v, a2d);
    clamped(p + 2 * n_ka, dc, n_k, wv, wd);
    clamped(p + 2 * n_ka + n_k, dc, n_k, nv, nd);
    T aw = a1v * a2v;
    T rad = inv_dx * (wd + aw * nd);
    T ad1 = inv_dtheta * a1d * a2v * nv;
    T ad2 = inv_dtheta * a1v * a2d * nv;
    V3<T> rXX = r1 * ad1 - r2 * ad2;
    V3<T> ddir = (rXX - u * dot(u, rXX)) * inv_dist;
    V3<T> dd = u * rad + ddir;
    st3(d1, -dd); st3(d1 + 3, u * ad1);
    st3(d2, dd); st3(d2 + 3, u * (-ad2));
    return wv + aw * nv;
}

template <class T> void quadspline_param_deriv(int n_ka, int n_k, T inv_dtheta, T inv_dx, const T* p, const T* x1,
                                               const T* x2, T* dp) {
    int np = 2 * n_ka + 2 * n_k;
    for (int i = 0; i < np; ++i) dp[i] = 0;
    V3<T> disp = ld3(x2) - ld3(x1), r1 = ld3(x1 + 3), r2 = ld3(x2 + 3);
    T dist2 = mag2(disp), inv_dist = T(1) / std::sqrt(dist2);
    T dc = dist2 * (inv_dist * inv_dx);
    V3<T> u = disp * inv_dist;
    T x1s = (dot(r1, u) + T(1)) * inv_dtheta + T(1), x2s = (-dot(r2, u) + T(1)) * inv_dtheta + T(1);
    T a1v, a1d, a2v, a2d, nv, nd;
    deboor(p, x1s, a1v, a1d);
    deboor(p + n_ka, x2s, a2v, a2d);
    clamped(p + 2 * n_ka + n_k, dc, n_k, nv, nd);
    T r[4];
    int sb = clamped_coeff_deriv(dc, n_k, r);
    for (int i = 0; i < 4; ++i) dp[2 * n_ka + sb + i] = r[i];
    for (int i = 0; i < 4; ++i) dp[2 * n_ka + n_k + sb + i] = a1v * a2v * r[i];
    sb = coeff_deriv(x1s, r);
    for (int i = 0; i < 4; ++i) dp[sb + i] = a2v * nv * r[i];
    sb = coeff_deriv(x2s, r);
    for (int i = 0; i < 4; ++i) dp[n_ka + sb + i] = a1v * nv * r[i];
}

enum IKind { IK_ROTAMER, IK_HBCOV, IK_PHB, IK_ENVCOV, IK_HBENV };

// Generic pair-interaction graph (InteractionGraph, src/interaction_graph.h:261-565)
template <class T> struct IGraph {
    IKind kind;
    bool symmetric;
    int d1, d2, n_param, n_type1, n_type2;
    vector<int> loc1, loc2, type1, type2, id1, id2;
    vector<T> param;
    T cutoff = 0;
    ExclRule rule;
    vector<T> x1, x2;  // packed positions
    vector<std::pair<int, int>> edges;
    vector<T> value, deriv, esens;  // deriv: per edge d1+d2 floats
    // candidate cache (src/interaction_graph.h:51-258): the pairs within
    // cutoff + buffer (buffer 1 + 0.2 cutoff, :396) at the positions of the
    // last rebuild, refined to the cutoff at every evaluation; rebuilt when an
    // element moved more than half the buffer since (:58-91).  The refined
    // list is the brute-force list at the cutoff, in the same order.
    vector<std::pair<int, int>> cand;
    vector<T> xc1, xc2;
    T cache_cutoff = 0;
    bool cache_valid = false;

    void load(const H5& h, IKind k) {
        kind = k;
        symmetric = (k == IK_ROTAMER);
        switch (k) {
            case IK_ROTAMER: d1 = 6; d2 = 6; n_param = 54; rule = EX_ROTAMER; break;
            case IK_HBCOV: d1 = 7; d2 = 6; n_param = 50; rule = EX_SEQ2; break;
            case IK_PHB: d1 = 6; d2 = 6; n_param = 8; rule = EX_SEQ1; break;
            case IK_ENVCOV: d1 = 6; d2 = 4; n_param = 4; rule = EX_SEQ2; break;
            case IK_HBENV: d1 = 6; d2 = 6; n_param = 4; rule = EX_SEQ2; break;
        }
        string s = symmetric ? "" : "1";
        loc1 = h.ri("index" + s);
        type1 = h.ri("type" + s);
        id1 = h.ri("id" + s);
        if (symmetric) {
            loc2 = loc1; type2 = type1; id2 = id1;
        } else {
            loc2 = h.ri("index2");
            type2 = h.ri("type2");
            id2 = h.ri("id2");
        }
        auto dm = h.dims("interaction_param");
        if (dm.size() != 3 || int(dm[2]) != n_param) throw Err("interaction_param shape mismatch");
        n_type1 = int(dm[0]);
        n_type2 = int(dm[1]);
        param = h.rf<T>("interaction_param");
        update_cutoff();
    }
    void update_cutoff() {
        // per-interaction cutoffs (src/bead_interaction.h:188-190, src/hbond.cpp:182-184,
        // :255-257, src/environment.cpp:118-120, :176-178); float arithmetic as written
        cutoff = 0;
        for (int a = 0; a < n_type1 * n_type2; ++a) {
            const T* p = &param[size_t(a) * n_param];
            T c = 0;
            switch (kind) {
                case IK_ROTAMER: c = T(float((12 - 2 - 1e-6) / double(1.f / 0.7f))); break;
                case IK_HBCOV: c = T(float((10 - 2 - 1e-6) / double(1.f / 0.625f))); break;
                case IK_PHB: c = T(std::sqrt(3.5f * 3.5f)); break;
                case IK_ENVCOV:
                case IK_HBENV: c = p[0] + T(1) / p[1]; break;
            }
            cutoff = std::max(cutoff, c);
        }
        cache_valid = false;
    }
    void gather(const Node<T>& n1, const Node<T>* n2) {
        x1.resize(3 * loc1.size());
        for (size_t i = 0; i < loc1.size(); ++i)
            for (int d = 0; d < 3; ++d) x1[3 * i + d] = n1.out[size_t(loc1[i]) * n1.width + d];
        const Node<T>& m = n2 ? *n2 : n1;
        x2.resize(3 * loc2.size());
        for (size_t i = 0; i < loc2.size(); ++i)
            for (int d = 0; d < 3; ++d) x2[3 * i + d] = m.out[size_t(loc2[i]) * m.width + d];
    }
    const T* P(int e) const {
        return &param[(size_t(type1[size_t(edges[size_t(e)].first)]) * n_type2 +
                       size_t(type2[size_t(edges[size_t(e)].second)])) * n_param];
    }
    // compute pair list, edge values and derivatives
    void compute(const Node<T>& n1, const Node<T>* n2) {
        gather(n1, n2);
        const vector<T>& y2 = symmetric ? x1 : x2;
        bool ok = cache_valid && xc1.size() == x1.size() && (symmetric || xc2.size() == x2.size());
        if (ok) {
            const T h = T(0.5f) * (cache_cutoff - cutoff), lim = h * h;
            auto moved = [&](const vector<T>& x, const vector<T>& xc) {
                for (size_t i = 0; i < x.size(); i += 3) {
                    T dx = x[i] - xc[i], dy = x[i + 1] - xc[i + 1], dz = x[i + 2] - xc[i + 2];
                    if (lim < dx * dx + dy * dy + dz * dz) return true;
                }
                return false;
            };
            ok = !moved(x1, xc1) && (symmetric || !moved(x2, xc2));
        }
        if (!ok) {
            cache_cutoff = cutoff + (T(1) + T(0.2f) * cutoff);
            find_pairs(symmetric, int(loc1.size()), int(loc2.size()), x1, y2, id1, id2, cache_cutoff, rule, cand);
            xc1 = x1;
            if (!symmetric) xc2 = x2;
            cache_valid = true;
        }
        // refine: the candidates within the cutoff now, in cache order
        // (src/interaction_graph.h:203-258), by find_pairs' own distance test
        edges.clear();
        const T c2 = cutoff * cutoff;
        for (const auto& pr : cand) {
            T dx = x1[3 * size_t(pr.first)] - y2[3 * size_t(pr.second)];
            T dy = x1[3 * size_t(pr.first) + 1] - y2[3 * size_t(pr.second) + 1];
            T dz = x1[3 * size_t(pr.first) + 2] - y2[3 * size_t(pr.second) + 2];
            T d2 = dx * dx + dy * dy + dz * dz;
            if (d2 < c2) edges.push_back(pr);
        }
        size_t ne = edges.size();
        value.assign(ne, T(0));
        deriv.assign(ne * size_t(d1 + d2), T(0));
        esens.assign(ne, T(0));
        const Node<T>& m = n2 ? *n2 : n1;
        // ProteinHBond evaluates lanes in groups of 4 edges: a group with no
        // edge inside the angular cutoff yields zeros (src/hbond.cpp:207-213)
        vector<char> group_active;
        if (kind == IK_PHB) group_active.assign((ne + 3) / 4, 0);
        for (int pass = (kind == IK_PHB ? 0 : 1); pass < 2; ++pass) {
            for (size_t e = 0; e < ne; ++e) {
                const T* a = &n1.out[size_t(loc1[size_t(edges[e].first)]) * n1.width];
                const T* b = &m.out[size_t(loc2[size_t(edges[e].second)]) * m.width];
                T* da = &deriv[e * size_t(d1 + d2)];
                T* db = da + d1;
                if (pass == 0) {
                    group_active[e / 4] |= phb_in_angle(a, b);
                    continue;
                }
                value[e] = edge(P(int(e)), a, b, da, db, kind == IK_PHB ? bool(group_active[e / 4]) : true);
            }
        }
    }
    static bool phb_in_angle(const T* H, const T* O) {
        V3<T> HO = ld3(H) - ld3(O);
        T m2 = mag2(HO) + T(1e-6f);
        V3<T> rHO = HO * (T(1) / std::sqrt(m2));
        return (dot(rHO, ld3(O + 3)) > T(0)) && (-dot(rHO, ld3(H + 3)) > T(0));
    }
    T edge(const T* p, const T* a, const T* b, T* da, T* db, bool active) const {
        switch (kind) {
            case IK_ROTAMER:
                return quadspline(15, 12, T(6), T(1.f / 0.7f), p, a, b, da, db);
            case IK_HBCOV: {
                // (src/hbond.cpp:258-280)
                T cov = quadspline(15, 10, T(6), T(1.f / 0.625f), p, a, b, da, db);
                T pre = (T(1) - a[6]) * (T(1) - a[6]);
                for (int i = 0; i < 6; ++i) { da[i] *= pre; db[i] *= pre; }
                da[6] = -cov * (T(1) - a[6]) * T(2);
                return pre * cov;
            }
            case IK_PHB: {
                // (src/hbond.cpp:164-236)
                V3<T> H = ld3(a), O = ld3(b), rHN = ld3(a + 3), rOC = ld3(b + 3);
                V3<T> HO = H - O;
                T m2 = mag2(HO) + T(1e-6f), inv = T(1) / std::sqrt(m2), mg = m2 * inv;
                V3<T> rHO = HO * inv;
                T dHOC = dot(rHO, rOC), dOHN = -dot(rHO, rHN);
                T hb = 0;
                V3<T> dH, drHN, drOC;
                if (active) {
                    T ov, od, iv, id_, a1v, a1d, a2v, a2d;
                    sigmoid((p[2] - mg) * p[3], ov, od);
                    sigmoid((mg - p[0]) * p[1], iv, id_);
                    T rv = ov * iv, rd = -p[3] * od * iv + p[1] * id_ * ov;
                    sigmoid((dHOC - p[4]) * p[5], a1v, a1d);
                    a1d *= p[5];
                    sigmoid((dOHN - p[4]) * p[5], a2v, a2d);
                    a2d *= p[5];
                    hb = rv * a1v * a2v;
                    T c0 = rd * a1v * a2v, c1 = rv * a1d * a2v, c2 = -rv * a1v * a2d;
                    drOC = rHO * c1;
                    drHN = rHO * c2;
                    dH = rHO * c0 + (rOC - rHO * dHOC) * (c1 * inv) + (rHN + rHO * dOHN) * (c2 * inv);
                }
                T hb_log = (T(1) <= hb) ? T(100) : -std::log(T(1) - hb);
                T pre = std::min(T(1) / (T(1) - hb), T(1e5f));
                st3(da, dH * pre); st3(da + 3, drHN * pre);
                st3(db, dH * (-pre)); st3(db + 3, drOC * pre);
                return hb_log;
            }
            case IK_ENVCOV: {
                // (src/environment.cpp:122-162)
                V3<T> disp = ld3(b) - ld3(a), r1 = ld3(a + 3);
                T prob = b[3];
                T d2 = mag2(disp), inv = T(1) / std::sqrt(d2), dist = d2 * inv;
                V3<T> u = disp * inv;
                T dp = dot(u, r1), rv, rd, av, ad;
                compact_sigmoid(dist - p[0], p[1], rv, rd);
                compact_sigmoid(p[2] - dp, p[3], av, ad);
                V3<T> dd = (u * (rd * av) - (r1 - u * dp) * (rv * ad * inv)) * prob;
                st3(da + 3, u * (-prob * rv * ad));
                st3(da, -dd);
                st3(db, dd);
                T score = rv * av;
                db[3] = score;
                return prob * score;
            }
            case IK_HBENV: {
                // (src/environment.cpp:180-220)
                V3<T> disp = ld3(b) - ld3(a), r1 = ld3(a + 3);
                T d2 = mag2(disp), inv = T(1) / std::sqrt(d2), dist = d2 * inv;
                V3<T> u = disp * inv;
                T dp = dot(u, r1), rv, rd, av, ad;
                compact_sigmoid(dist - p[0], p[1], rv, rd);
                compact_sigmoid(p[2] - dp, p[3], av, ad);
                V3<T> dd = u * (rd * av) - (r1 - u * dp) * (rv * ad * inv);
                st3(da + 3, u * (-rv * ad));
                st3(da, -dd);
                st3(db, dd);
                return rv * av;
            }
        }
        return 0;
    }
    // scatter sensitivities back to the input nodes (src/interaction_graph.h:511-564)
    void propagate(Node<T>& n1, Node<T>* n2) {
        Node<T>& m = n2 ? *n2 : n1;
        for (size_t e = 0; e < edges.size(); ++e) {
            T s = esens[e];
            const T* da = &deriv[e * size_t(d1 + d2)];
            const T* db = da + d1;
            T* s1 = &n1.sens[size_t(loc1[size_t(edges[e].first)]) * n1.width];
            T* s2 = &m.sens[size_t(loc2[size_t(edges[e].second)]) * m.width];
            for (int d = 0; d < d1; ++d) s1[d] += s * da[d];
            for (int d = 0; d < d2; ++d) s2[d] += s * db[d];
        }
    }
    // dE/dparam accumulated per type pair with the current edge sensitivities
    // (src/interaction_graph.h:406-416, :498-506, :542-550)
    vector<float> param_deriv(const Node<T>& n1, const Node<T>* n2) const {
        vector<double> acc(param.size(), 0.);
        const Node<T>& m = n2 ? *n2 : n1;
        vector<T> dp(static_cast<size_t>(n_param));
        for (size_t e = 0; e < edges.size(); ++e) {
            const T* a = &n1.out[size_t(loc1[size_t(edges[e].first)]) * n1.width];
            const T* b = &m.out[size_t(loc2[size_t(edges[e].second)]) * m.width];
            const T* p = P(int(e));
            if (kind == IK_ROTAMER) {
                quadspline_param_deriv(15, 12, T(6), T(1.f / 0.7f), p, a, b, dp.data());
            } else if (kind == IK_HBCOV) {
                quadspline_param_deriv(15, 10, T(6), T(1.f / 0.625f), p, a, b, dp.data());
                T pre = (T(1) - a[6]) * (T(1) - a[6]);
                for (auto& x : dp) x *= pre;
            } else {
                std::fill(dp.begin(), dp.end(), T(0));
            }
            int t1 = type1[size_t(edges[e].first)], t2 = type2[size_t(edges[e].second)];
            for (int k = 0; k < n_param; ++k) {
                acc[(size_t(t1) * n_type2 + t2) * n_param + k] += double(esens[e] * dp[size_t(k)]);
                if (symmetric) acc[(size_t(t2) * n_type1 + t1) * n_param + k] += double(esens[e] * dp[size_t(k)]);
            }
        }
        return vector<float>(acc.begin(), acc.end());
    }
};

// protein_hbond: per-donor/acceptor hbond score in multiplicative space
// (ProteinHBond, src/hbond.cpp:357-435)
template <class T> struct ProteinHBondNode : Node<T> {
    IGraph<T> g;
    int n_don, n_acc;
    ProteinHBondNode(const H5& h) {
        g.load(h, IK_PHB);
        n_don = int(g.loc1.size());
        n_acc = int(g.loc2.size());
        this->alloc(n_don + n_acc, 7);
    }
    void forward(Engine<T>& e, bool) override {
        auto& in = e.arg(*this, 0);
        for (int i = 0; i < this->n_elem; ++i) {
            for (int d = 0; d < 6; ++d) this->out[7 * size_t(i) + d] = in.out[6 * size_t(i) + d];
            this->out[7 * size_t(i) + 6] = 0;
        }
        g.compute(in, &in);
        for (size_t k = 0; k < g.edges.size(); ++k) {
            this->out[7 * size_t(g.edges[k].first) + 6] += g.value[k];
            this->out[7 * size_t(g.edges[k].second + n_don) + 6] += g.value[k];
        }
        for (int i = 0; i < this->n_elem; ++i) this->out[7 * size_t(i) + 6] = T(1) - std::exp(-this->out[7 * size_t(i) + 6]);
    }
    void backward(Engine<T>& e) override {
        auto& in = e.arg(*this, 0);
        vector<T> ss(static_cast<size_t>(this->n_elem));
        for (int i = 0; i < this->n_elem; ++i) ss[size_t(i)] = this->sens[7 * size_t(i) + 6] * (T(1) - this->out[7 * size_t(i) + 6]);
        for (size_t k = 0; k < g.edges.size(); ++k) g.esens[k] = ss[size_t(g.edges[k].first)] + ss[size_t(g.edges[k].second + n_don)];
        g.propagate(in, &in);
        for (int i = 0; i < this->n_elem; ++i) {
            int l = i < n_don ? g.loc1[size_t(i)] : g.loc2[size_t(i - n_don)];
            for (int d = 0; d < 6; ++d) in.sens[6 * size_t(l) + d] += this->sens[7 * size_t(i) + d];
        }
    }
    const vector<std::pair<int, int>>* edges() const override { return &g.edges; }
};

// hbond_coverage(+_hydrophobe): sum of coverage per side-chain bead (HBondCoverage, src/hbond.cpp:438-484)
template <class T> struct HBCoverageNode : Node<T> {
    IGraph<T> g;
    HBCoverageNode(const H5& h) {
        g.load(h, IK_HBCOV);
        this->alloc(int(g.loc2.size()), 1);
    }
    void forward(Engine<T>& e, bool) override {
        g.compute(e.arg(*this, 0), &e.arg(*this, 1));
        std::fill(this->out.begin(), this->out.end(), T(0));
        for (size_t k = 0; k < g.edges.size(); ++k) this->out[size_t(g.edges[k].second)] += g.value[k];
    }
    void backward(Engine<T>& e) override {
        for (size_t k = 0; k < g.edges.size(); ++k) g.esens[k] = this->sens[size_t(g.edges[k].second)];
        g.propagate(e.arg(*this, 0), &e.arg(*this, 1));
    }
    vector<float> get_param() override { return vector<float>(g.param.begin(), g.param.end()); }
    void set_param(const vector<float>& p) override {
        if (p.size() != g.param.size()) throw Err("Bad param size");
        g.param.assign(p.begin(), p.end());
        g.update_cutoff();
    }
    vector<float> param_deriv(Engine<T>& e) override { return g.param_deriv(e.arg(*this, 0), &e.arg(*this, 1)); }
    vector<float> value_by_name(const string& w) override {
        if (w == "count_edges_by_type") return count_edges(g);
        return Node<T>::value_by_name(w);
    }
    static vector<float> count_edges(const IGraph<T>& g) {
        vector<float> r(size_t(g.n_type1 * g.n_type2), 0.f);
        for (auto& ed : g.edges) r[size_t(g.type1[size_t(ed.first)] * g.n_type2 + g.type2[size_t(ed.second)])] += 1.f;
        return r;
    }
    const vector<std::pair<int, int>>* edges() const override { return &g.edges; }
};

// environment_coverage: CB (or H/O) coverage by weighted beads, per amino-acid
// type of the bead's residue (EnvironmentCoverage, src/environment.cpp:288-348)
template <class T> struct EnvCoverageNode : Node<T> {
    IGraph<T> g;
    int n_aa;
    vector<int> aa;
    EnvCoverageNode(const H5& h) {
        g.load(h, IK_ENVCOV);
        n_aa = int(h.attr("num_aa_types"));
        aa = h.ri("aa_types");
        this->alloc(int(g.loc1.size()) * n_aa, 1);
    }
    size_t slot(size_t k) const { return size_t(g.edges[k].first) * n_aa + size_t(aa[size_t(g.id2[size_t(g.edges[k].second)])]); }
    void forward(Engine<T>& e, bool) override {
        g.compute(e.arg(*this, 0), &e.arg(*this, 1));
        std::fill(this->out.begin(), this->out.end(), T(0));
        for (size_t k = 0; k < g.edges.size(); ++k) this->out[slot(k)] += g.value[k];
    }
    void backward(Engine<T>& e) override {
        for (size_t k = 0; k < g.edges.size(); ++k) g.esens[k] = this->sens[slot(k)];
        g.propagate(e.arg(*this, 0), &e.arg(*this, 1));
    }
    const vector<std::pair<int, int>>* edges() const override { return &g.edges; }
};

// hb_environment_coverage: H/O coverage (HbondEnvironmentCoverage, src/environment.cpp:350-385)
template <class T> struct HBEnvCoverageNode : Node<T> {
    IGraph<T> g;
    HBEnvCoverageNode(const H5& h) {
        g.load(h, IK_HBENV);
        this->alloc(int(g.loc1.size()), 1);
    }
    void forward(Engine<T>& e, bool) override {
        g.compute(e.arg(*this, 0), &e.arg(*this, 1));
        std::fill(this->out.begin(), this->out.end(), T(0));
        for (size_t k = 0; k < g.edges.size(); ++k) this->out[size_t(g.edges[k].first)] += g.value[k];
    }
    void backward(Engine<T>& e) override {
        for (size_t k = 0; k < g.edges.size(); ++k) g.esens[k] = this->sens[size_t(g.edges[k].first)];
        g.propagate(e.arg(*this, 0), &e.arg(*this, 1));
    }
    const vector<std::pair<int, int>>* edges() const override { return &g.edges; }
};

// sigmoid_coupling environment energy (SigmoidCoupling, src/environment.cpp:851-1003)
template <class T> struct SigmoidCouplingNode : Node<T> {
    vector<T> scale, center, sharp, weights;
    vector<int> ctype;
    int n_rt, n_res;
    SigmoidCouplingNode(const H5& h) {
        this->potential_node = true;
        scale = h.rf<T>("scale");
        center = h.rf<T>("center");
        sharp = h.rf<T>("sharpness");
        weights = h.rf<T>("weights");
        ctype = h.ri("coupling_types");
        n_rt = int(scale.size());
        n_res = int(ctype.size());
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& in = e.arg(*this, 0);
        T pot = 0;
        for (int r = 0; r < n_res; ++r) {
            int c = ctype[size_t(r)];
            T wn = 0;
            for (int a = 0; a < n_rt; ++a) wn += weights[size_t(c) * n_rt + a] * in.out[size_t(r) * n_rt + a];
            T v, d;
            compact_sigmoid(wn - center[size_t(c)], sharp[size_t(c)], v, d);
            pot += scale[size_t(c)] * v;
            for (int a = 0; a < n_rt; ++a) in.sens[size_t(r) * n_rt + a] += weights[size_t(c) * n_rt + a] * scale[size_t(c)] * d;
        }
        this->pot = energy ? pot : T(0);
    }
};

// nonlinear_coupling environment energy, clamped spline of the weighted
// coverage (NonlinearCoupling, src/environment.cpp:701-849)
template <class T> struct NonlinearCouplingNode : Node<T> {
    vector<T> coeff, weights;
    vector<int> ctype;
    int n_rt, n_coeff, n_res, n_indep;
    T offset, inv_dx;
    NonlinearCouplingNode(const H5& h) {
        this->potential_node = true;
        coeff = h.rf<T>("coeff");
        auto d = h.dims("coeff");
        n_rt = int(d[0]);
        n_coeff = int(d[1]);
        weights = h.rf<T>("weights");
        ctype = h.ri("coupling_types");
        n_res = int(ctype.size());
        offset = T(h.attr("spline_offset", NAN, "coeff"));
        inv_dx = T(h.attr("spline_inv_dx", NAN, "coeff"));
        n_indep = int(h.attr("number_independent_weights"));
    }
    T wnum(Engine<T>& e, int r) {
        auto& in = e.arg(*this, 0);
        int c = ctype[size_t(r)];
        T wn = 0;
        for (int a = 0; a < n_rt; ++a) wn += weights[size_t(c) * n_rt + a] * in.out[size_t(r) * n_rt + a];
        return wn;
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& in = e.arg(*this, 0);
        T pot = 0;
        for (int r = 0; r < n_res; ++r) {
            int c = ctype[size_t(r)];
            T v, d;
            clamped(&coeff[size_t(c) * n_coeff], (wnum(e, r) - offset) * inv_dx, n_coeff, v, d);
            pot += v;
            for (int a = 0; a < n_rt; ++a) in.sens[size_t(r) * n_rt + a] = weights[size_t(c) * n_rt + a] * inv_dx * d;
        }
        this->pot = energy ? pot : T(0);
    }
    vector<float> get_param() override {
        vector<float> p(coeff.begin(), coeff.end());
        p.insert(p.end(), weights.begin(), weights.end());
        return p;
    }
    void set_param(const vector<float>& p) override {
        if (p.size() != coeff.size() + weights.size()) throw Err("Bad param size");
        for (size_t i = 0; i < coeff.size(); ++i) coeff[i] = p[i];
        for (size_t i = 0; i < weights.size(); ++i) weights[i] = p[coeff.size() + i];
    }
    vector<float> param_deriv(Engine<T>& e) override {
        auto& in = e.arg(*this, 0);
        vector<double> d(coeff.size() + weights.size(), 0.);
        vector<T> sens(size_t(n_res), T(0));
        for (int r = 0; r < n_res; ++r) {
            int c = ctype[size_t(r)];
            T x = (wnum(e, r) - offset) * inv_dx, res[4];
            int sb = clamped_coeff_deriv(x, n_coeff, res);
            for (int i = 0; i < 4; ++i) d[size_t(c) * n_coeff + size_t(sb + i)] += double(res[i]);
            if (n_indep > 1) {
                T v, dv;
                clamped(&coeff[size_t(c) * n_coeff], x, n_coeff, v, dv);
                sens[size_t(r)] = inv_dx * dv;
            }
        }
        if (n_indep > 1) {
            size_t cs = coeff.size();
            for (int r = 0; r < n_res; ++r) {
                int c = ctype[size_t(r)];
                for (int a = 0; a < n_rt; ++a) {
                    double da = double(sens[size_t(r)] * in.out[size_t(r) * n_rt + a]);
                    if (n_indep == 400) d[cs + size_t(c) * n_rt + a] += da;
                    else if (n_indep == 20)
                        for (int a2 = 0; a2 < n_rt; ++a2) d[cs + size_t(a2) * n_rt + a] += da;
                }
            }
        }
        return vector<float>(d.begin(), d.end());
    }
};

// bb_sigmoid_coupling (BackboneSigmoidCoupling, src/environment.cpp:1054-1138)
template <class T> struct BBSigmoidNode : Node<T> {
    vector<T> weights;
    int n_rt;
    T scale, center, sharp, hbw;
    BBSigmoidNode(const H5& h) {
        this->potential_node = true;
        weights = h.rf<T>("weights");
        n_rt = int(h.attr("num_aa_types"));
        scale = T(float(h.attr("scale")));
        center = T(float(h.attr("center")));
        sharp = T(float(h.attr("sharpness")));
        hbw = T(float(h.attr("hbond_weight")));
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& sc = e.arg(*this, 0);
        auto& hb = e.arg(*this, 1);
        int n_bb = sc.n_elem / n_rt;
        T pot = 0;
        for (int r = 0; r < n_bb; ++r) {
            T bl = 0;
            for (int a = 0; a < n_rt; ++a) bl += weights[size_t(a)] * sc.out[size_t(r) * n_rt + a];
            bl += hbw * hb.out[size_t(r)];
            T v, d;
            compact_sigmoid(bl - center, sharp, v, d);
            pot += scale * v;
            T dp = scale * d;
            for (int a = 0; a < n_rt; ++a) sc.sens[size_t(r) * n_rt + a] += weights[size_t(a)] * dp;
            hb.sens[size_t(r)] += hbw * dp;
        }
        this->pot = energy ? pot : T(0);
    }
};

// hbond_energy: helix/sheet/turn energies times hbond counts (HBondEnergy, src/hbond.cpp:487-739)
template <class T> struct HBondEnergyNode : Node<T> {
    vector<T> prm;
    vector<int> dres, ares;
    int n_res;
    HBondEnergyNode(const H5& h) {
        this->potential_node = true;
        prm = h.rf<T>("parameters");
        dres = h.ri("donor_resid");
        ares = h.ri("acceptor_resid");
        n_res = int(h.dims("rama_resid")[0]);
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& pp = e.arg(*this, 0);
        auto& ra = e.arg(*this, 1);
        int nd = int(dres.size());
        vector<T> E(static_cast<size_t>(n_res)), dphi(static_cast<size_t>(n_res)), dpsi(static_cast<size_t>(n_res));
        for (int i = 0; i < n_res; ++i) {
            T phi = ra.out[2 * size_t(i)], psi = ra.out[2 * size_t(i) + 1];
            T p1v, p1d, p2v, p2d, s1v, s1d, s2v, s2d;
            compact_sigmoid(phi - prm[4], prm[5], p1v, p1d);
            compact_sigmoid(phi - prm[6], prm[7], p2v, p2d);
            compact_sigmoid(psi - prm[8], prm[9], s1v, s1d);
            compact_sigmoid(psi - prm[10], prm[11], s2v, s2d);
            T turn = (T(1) - p1v) * p2v, psis = (T(1) - s1v) * s2v;
            T nturn = T(1) - turn, npsi = T(1) - psis;
            T helix = nturn * psis, sheet = nturn * npsi;
            T dturn = p2d - (p1d * p2v + p1v * p2d);
            T dpsis = s2d - (s1d * s2v + s1v * s2d);
            E[size_t(i)] = prm[0] * helix + prm[1] * sheet + prm[2] * turn;
            dphi[size_t(i)] = prm[0] * (-dturn * psis) + prm[1] * (-dturn * npsi) + prm[2] * dturn;
            dpsi[size_t(i)] = prm[0] * (nturn * dpsis) + prm[1] * (nturn * -dpsis);
        }
        vector<T> hb1(size_t(n_res), T(0)), hb2(size_t(std::max(n_res - 1, 0)), T(0));
        std::map<int, int> rd, racc;
        for (int k = 0; k < nd; ++k) { rd.emplace(dres[size_t(k)], k); hb1[size_t(dres[size_t(k)])] += pp.out[7 * size_t(k) + 6]; }
        for (size_t k = 0; k < ares.size(); ++k) { racc.emplace(ares[k], int(k)); hb1[size_t(ares[k])] += pp.out[7 * (k + size_t(nd)) + 6]; }
        for (int k = 0; k < nd; ++k) hb2[size_t(dres[size_t(k)] - 1)] += pp.out[7 * size_t(k) + 6];
        for (size_t k = 0; k < ares.size(); ++k) hb2[size_t(ares[k])] += pp.out[7 * (k + size_t(nd)) + 6];
        T pot = 0;
        for (int i = 0; i < n_res; ++i) {
            if (hb1[size_t(i)] == T(0)) continue;
            pot += hb1[size_t(i)] * E[size_t(i)];
            auto it = rd.find(i);
            if (it != rd.end()) pp.sens[7 * size_t(it->second) + 6] += E[size_t(i)];
            it = racc.find(i);
            if (it != racc.end()) pp.sens[7 * size_t(it->second + nd) + 6] += E[size_t(i)];
            ra.sens[2 * size_t(i)] += hb1[size_t(i)] * dphi[size_t(i)];
            ra.sens[2 * size_t(i) + 1] += hb1[size_t(i)] * dpsi[size_t(i)];
        }
        for (int i = 0; i < n_res - 1; ++i) {
            if (hb2[size_t(i)] <= T(1)) continue;
            T v, d;
            compact_sigmoid(T(1.5) - hb2[size_t(i)], T(2), v, d);
            pot += v * prm[3];
            T dE = -d * prm[3];
            auto it = rd.find(i + 1);
            if (it != rd.end()) pp.sens[7 * size_t(it->second) + 6] += dE;
            it = racc.find(i);
            if (it != racc.end()) pp.sens[7 * size_t(it->second + nd) + 6] += dE;
        }
        this->pot = energy ? pot : T(0);
    }
};

// backbone steric repulsion between rigid residues (BackbonePairs, src/backbone_steric.cpp:38-147)
template <class T> struct BackbonePairsNode : Node<T> {
    vector<int> res, nat;
    vector<T> refp;  // (n,4,3)
    BackbonePairsNode(const H5& h) {
        this->potential_node = true;
        res = h.ri("id");
        nat = h.ri("n_atom");
        refp = h.rf<T>("ref_pos");
    }
    void forward(Engine<T>& e, bool energy) override {
        auto& af = e.arg(*this, 0);
        int n = int(res.size());
        vector<V3<T>> x(static_cast<size_t>(4 * n)), t(static_cast<size_t>(n));
        for (int r = 0; r < n; ++r) {
            const T* a = &af.out[7 * size_t(res[size_t(r)])];
            T U[9];
            quat_to_rot(a + 3, U);
            t[size_t(r)] = V3<T>(a[0], a[1], a[2]);
            for (int k = 0; k < nat[size_t(r)]; ++k) x[4 * size_t(r) + k] = rot(U, ld3(&refp[(size_t(r) * 4 + k) * 3])) + t[size_t(r)];
        }
        const T c2 = T(3.f * 3.f + 0.1f * 3.f);
        T pot = 0;
        for (int i = 0; i < n; ++i)
            for (int j = i + 1; j < n; ++j) {
                if (!acceptable(EX_SEQ1, res[size_t(i)], res[size_t(j)])) continue;
                V3<T> di, ti, dj, tj;
                bool hit = false;
                for (int a = 0; a < nat[size_t(i)]; ++a)
                    for (int b = 0; b < nat[size_t(j)]; ++b) {
                        V3<T> r = x[4 * size_t(i) + a] - x[4 * size_t(j) + b];
                        T m2 = mag2(r);
                        if (m2 > c2) continue;
                        hit = true;
                        T v, d;
                        compact_sigmoid(m2 - T(9), T(1.f / (3.0f * 0.10f)), v, d);
                        if (energy) pot += T(4) * v;
                        V3<T> g = r * (T(2) * T(4) * d);
                        di += g; ti += cross(x[4 * size_t(i) + a] - t[size_t(i)], g);
                        dj -= g; tj += cross(x[4 * size_t(j) + b] - t[size_t(j)], -g);
                    }
                if (hit) {
                    T* si = &af.sens[7 * size_t(res[size_t(i)])];
                    T* sj = &af.sens[7 * size_t(res[size_t(j)])];
                    add3(si, di); add3(si + 3, ti);
                    add3(sj, dj); add3(sj + 3, tj);
                }
            }
        this->pot = energy ? pot : T(0);
    }
};

// ----------------------------------------------------------- rotamer BP ---
// Side-chain rotamer node: loopy belief propagation over residue rotamer
// states (RotamerSidechain, src/rotamer.cpp:628-1169).
template <class T> struct RotamerNode : Node<T> {
    IGraph<T> g;
    int n_prob;
    T damping, tol;
    int max_iter, chunk;
    long n_bad_solve = 0;
    int last_iter = 0;
    // node classes
    struct NodeSet {
        int n_rot = 0, n = 0;
        vector<T> E1, prob, cur, old, eoff;  // n x n_rot
    };
    NodeSet ns[7];
    // residue-pair edges by class
    struct EdgeSet {
        int r1 = 0, r2 = 0;
        vector<int> a, b;           // node local indices
        vector<T> prob;             // n x r1*r2 (product of exp(-E))
        vector<T> cur, old;         // n x (r1 + r2): message into node a, into node b
        vector<T> marg;             // n x r1*r2
        std::map<std::pair<int, int>, int> loc;
        vector<std::pair<int, int>> bead_loc;  // (bead edge, dim) with edge index
        vector<int> bead_edge_ix;
    };
    EdgeSet es[7][7];
    vector<int> bead_rot, bead_nrot, bead_res;  // decoded ids per bead (in igraph order)

    RotamerNode(const H5& h) {
        this->potential_node = true;
        H5 hp{h.f, h.p("pair_interaction")};
        g.load(hp, IK_ROTAMER);
        damping = T(float(h.attr("damping")));
        max_iter = int(h.attr("max_iter"));
        tol = T(float(h.attr("tol")));
        chunk = int(h.attr("iteration_chunk_size"));
        std::map<int, std::set<int>> uniq;
        for (int id : g.id1) {
            int rot = id & 15, nr = (id >> 4) & 15, res = id >> 8;
            if (rot >= nr) throw Err("invalid rotamer number");
            if (nr != 1 && nr != 3 && nr != 6) throw Err("unsupported rotamer count");
            bead_rot.push_back(rot);
            bead_nrot.push_back(nr);
            bead_res.push_back(res);
            uniq[nr].insert(res);
        }
        for (int r : {1, 3, 6}) {
            ns[r].n_rot = r;
            ns[r].n = int(uniq[r].size());
        }
        for (int a : {1, 3, 6})
            for (int b : {1, 3, 6})
                if (a <= b) { es[a][b].r1 = a; es[a][b].r2 = b; }
    }

    static T node_free_energy(const NodeSet& s, int i) {
        const T* b = &s.cur[size_t(i) * s.n_rot];
        const T* pr = &s.prob[size_t(i) * s.n_rot];
        T sum = 0;
        for (int k = 0; k < s.n_rot; ++k) sum += b[k];
        T en = s.eoff[size_t(i)];
        for (int k = 0; k < s.n_rot; ++k) {
            T bk = b[k] / sum;
            en += bk * std::log((T(1e-10f) + bk) / (T(1e-10f) + pr[k]));
        }
        return en;
    }
    T edge_free_energy(const EdgeSet& E, int e) {
        const T* b1 = &ns[E.r1].cur[size_t(E.a[size_t(e)]) * E.r1];
        const T* b2 = &ns[E.r2].cur[size_t(E.b[size_t(e)]) * E.r2];
        const T* p = &E.marg[size_t(e) * E.r1 * E.r2];
        const T* pr = &E.prob[size_t(e) * E.r1 * E.r2];
        T en = 0;
        for (int i = 0; i < E.r1; ++i)
            for (int j = 0; j < E.r2; ++j) {
                int k = i * E.r2 + j;
                en += p[k] * std::log((T(1e-10f) + p[k]) / (T(1e-10f) + pr[k] * b1[i] * b2[j]));
            }
        return en;
    }

    void fill(Engine<T>& e) {
        // node energies from the 1-body inputs (src/rotamer.cpp:854-884)
        for (int r : {1, 3, 6}) {
            ns[r].E1.assign(size_t(ns[r].n) * r, T(0));
            ns[r].cur.assign(size_t(ns[r].n) * r, T(0));
            ns[r].old.assign(size_t(ns[r].n) * r, T(0));
        }
        for (size_t n = 0; n < g.loc1.size(); ++n) {
            T en = 0;
            for (int k = 0; k < n_prob_nodes(); ++k) {
                auto& pn = e.arg(*this, 1 + k);
                en += pn.out[size_t(g.loc1[n]) * pn.width];
            }
            ns[bead_nrot[n]].E1[size_t(bead_res[n]) * bead_nrot[n] + size_t(bead_rot[n])] += en;
        }
        for (int r : {1, 3, 6}) {
            auto& s = ns[r];
            s.prob.assign(size_t(s.n) * r, T(0));
            s.eoff.assign(size_t(s.n), T(0));
            for (int i = 0; i < s.n; ++i) {
                T m = s.E1[size_t(i) * r];
                for (int k = 1; k < r; ++k) m = std::min(m, s.E1[size_t(i) * r + k]);
                for (int k = 0; k < r; ++k) s.prob[size_t(i) * r + k] = std::exp(m - s.E1[size_t(i) * r + k]);
                s.eoff[size_t(i)] = m;
            }
        }
        // edge probabilities (src/rotamer.cpp:886-912)
        g.compute(e.arg(*this, 0), nullptr);
        for (int a : {1, 3, 6})
            for (int b : {1, 3, 6})
                if (a <= b) {
                    auto& E = es[a][b];
                    E.a.clear(); E.b.clear(); E.prob.clear(); E.loc.clear(); E.bead_loc.clear(); E.bead_edge_ix.clear();
                }
        for (size_t k = 0; k < g.edges.size(); ++k) {
            int u = g.edges[k].first, v = g.edges[k].second;
            if (bead_nrot[size_t(u)] > bead_nrot[size_t(v)]) std::swap(u, v);
            int r1 = bead_nrot[size_t(u)], r2 = bead_nrot[size_t(v)];
            auto& E = es[r1][r2];
            auto key = std::make_pair(bead_res[size_t(u)], bead_res[size_t(v)]);
            auto it = E.loc.find(key);
            int ix;
            if (it == E.loc.end()) {
                ix = int(E.a.size());
                E.loc[key] = ix;
                E.a.push_back(key.first);
                E.b.push_back(key.second);
                E.prob.resize(E.prob.size() + size_t(r1 * r2), T(1));
            } else {
                ix = it->second;
            }
            int dim = bead_rot[size_t(u)] * r2 + bead_rot[size_t(v)];
            E.prob[size_t(ix) * r1 * r2 + dim] *= std::exp(-g.value[k]);
            E.bead_loc.emplace_back(int(k), dim);
            E.bead_edge_ix.push_back(ix);
        }
        // 1-rotamer edges fold into the partner's node probabilities (src/rotamer.cpp:398-405)
        for (int r2 : {3, 6}) {
            auto& E = es[1][r2];
            for (size_t ix = 0; ix < E.a.size(); ++ix)
                for (int k = 0; k < r2; ++k) ns[r2].prob[size_t(E.b[ix]) * r2 + k] *= E.prob[ix * r2 + k];
        }
    }
    int n_prob_nodes() const { return int(this->args.size()) - 1; }

    void update(EdgeSet& E) {
        // one synchronous BP sweep over the edges of a class (EdgeHolder::update_beliefs,
        // src/rotamer.cpp:500-569)
        auto& A = ns[E.r1];
        auto& B = ns[E.r2];
        int r1 = E.r1, r2 = E.r2, w = r1 + r2;
        for (size_t e = 0; e < E.a.size(); ++e) {
            const T* oa = &A.old[size_t(E.a[e]) * r1];
            const T* ob = &B.old[size_t(E.b[e]) * r2];
            const T* om = &E.old[e * w];
            T v1[6], v2[6], m1[6], m2[6];
            for (int i = 0; i < r1; ++i) v1[i] = oa[i] / (T(1e-10f) + om[i]);
            for (int j = 0; j < r2; ++j) v2[j] = ob[j] / (T(1e-10f) + om[r1 + j]);
            const T* P = &E.prob[e * r1 * r2];
            for (int i = 0; i < r1; ++i) {
                T s = 0;
                for (int j = 0; j < r2; ++j) s += P[i * r2 + j] * v2[j];
                m1[i] = s;
            }
            for (int j = 0; j < r2; ++j) {
                T s = 0;
                for (int i = 0; i < r1; ++i) s += P[i * r2 + j] * v1[i];
                m2[j] = s;
            }
            T* ca = &A.cur[size_t(E.a[e]) * r1];
            T* cb = &B.cur[size_t(E.b[e]) * r2];
            T sa = 0, sb = 0;
            for (int i = 0; i < r1; ++i) { ca[i] *= m1[i]; sa += ca[i]; }
            for (int j = 0; j < r2; ++j) { cb[j] *= m2[j]; sb += cb[j]; }
            for (int i = 0; i < r1; ++i) ca[i] *= T(1) / sa;
            for (int j = 0; j < r2; ++j) cb[j] *= T(1) / sb;
            // messages, each L1-normalised
            T s1 = 0, s2 = 0;
            for (int i = 0; i < r1; ++i) s1 += m1[i];
            for (int j = 0; j < r2; ++j) s2 += m2[j];
            T* cm = &E.cur[e * w];
            for (int i = 0; i < r1; ++i) cm[i] = m1[i] * (T(1) / s1);
            for (int j = 0; j < r2; ++j) cm[r1 + j] = m2[j] * (T(1) / s2);
        }
    }
    void standardize(NodeSet& s, T d) {
        // (NodeHolder::standardize_belief_update, src/rotamer.cpp:259-273)
        for (int i = 0; i < s.n; ++i) {
            T* b = &s.cur[size_t(i) * s.n_rot];
            const T* o = &s.old[size_t(i) * s.n_rot];
            T m = b[0];
            for (int k = 1; k < s.n_rot; ++k) m = std::max(m, b[k]);
            T inv = T(1) / m;
            for (int k = 0; k < s.n_rot; ++k) b[k] = d != T(0) ? (T(1) - d) * inv * b[k] + d * o[k] : inv * b[k];
        }
    }
    void new_beliefs(T d, bool swap_initial) {
        // (calculate_new_beliefs, src/rotamer.cpp:1089-1103)
        ns[3].cur = ns[3].prob;
        ns[6].cur = ns[6].prob;
        update(es[3][3]);
        update(es[3][6]);
        update(es[6][6]);
        if (swap_initial) { std::swap(ns[3].cur, ns[3].old); std::swap(ns[6].cur, ns[6].old); }
        standardize(ns[3], d);
        standardize(ns[6], d);
    }
    T max_dev(const NodeSet& s) {
        T dev = 0;
        for (size_t i = 0; i < s.cur.size(); ++i) dev = std::max(s.cur[i] - s.old[i], dev);
        return dev;
    }
    void solve() {
        // (solve_for_marginals, src/rotamer.cpp:1106-1162)
        for (int r : {1, 3, 6}) ns[r].old = ns[r].prob;
        for (int a : {3, 6})
            for (int b : {3, 6})
                if (a <= b) {
                    auto& E = es[a][b];
                    E.old.assign(E.a.size() * size_t(a + b), T(1));
                    E.cur.assign(E.a.size() * size_t(a + b), T(0));
                }
        new_beliefs(T(0), true);
        T dev = T(1e10f);
        int iter = 0;
        for (; dev > tol && iter < max_iter; iter += chunk) {
            for (int j = 0; j < chunk; ++j) {
                std::swap(ns[3].cur, ns[3].old);
                std::swap(ns[6].cur, ns[6].old);
                for (auto* E : {&es[3][3], &es[3][6], &es[6][6]}) std::swap(E->cur, E->old);
                new_beliefs(damping, false);
            }
            dev = std::max(max_dev(ns[3]), max_dev(ns[6]));
        }
        last_iter = iter;
        if (iter >= max_iter - chunk - 1) n_bad_solve++;
        // marginals (src/rotamer.cpp:283-290, :425-449)
        ns[1].cur.assign(ns[1].prob.size(), T(1));
        for (int r : {3, 6}) {
            auto& s = ns[r];
            for (int i = 0; i < s.n; ++i) {
                T sum = 0;
                for (int k = 0; k < r; ++k) sum += s.cur[size_t(i) * r + k];
                for (int k = 0; k < r; ++k) s.cur[size_t(i) * r + k] *= T(1) / sum;
            }
        }
        for (auto* Ep : {&es[3][3], &es[3][6], &es[6][6]}) {
            auto& E = *Ep;
            int r1 = E.r1, r2 = E.r2, w = r1 + r2;
            E.marg.assign(E.a.size() * size_t(r1 * r2), T(0));
            for (size_t e = 0; e < E.a.size(); ++e) {
                const T* b1 = &ns[r1].cur[size_t(E.a[e]) * r1];
                const T* b2 = &ns[r2].cur[size_t(E.b[e]) * r2];
                const T* m = &E.cur[e * w];
                T* mg = &E.marg[e * size_t(r1 * r2)];
                T s = 0;
                for (int i = 0; i < r1; ++i)
                    for (int j = 0; j < r2; ++j) {
                        T v = E.prob[e * size_t(r1 * r2) + size_t(i * r2 + j)] * (b1[i] / (T(1e-10f) + m[i])) *
                              (b2[j] / (T(1e-10f) + m[r1 + j]));
                        mg[i * r2 + j] = v;
                        s += v;
                    }
                for (int k = 0; k < r1 * r2; ++k) mg[k] *= T(1) / s;
            }
        }
    }
    void forward(Engine<T>& e, bool energy) override {
        fill(e);
        solve();
        // sensitivities (src/rotamer.cpp:1057-1086)
        for (int a : {1, 3, 6})
            for (int b : {1, 3, 6})
                if (a <= b) {
                    auto& E = es[a][b];
                    for (size_t k = 0; k < E.bead_loc.size(); ++k) {
                        int be = E.bead_loc[k].first, dim = E.bead_loc[k].second, ix = E.bead_edge_ix[k];
                        T s;
                        if (a == 1 && b == 1) s = 1;
                        else if (a == 1) s = ns[b].cur[size_t(E.b[size_t(ix)]) * b + size_t(dim)];
                        else s = E.marg[size_t(ix) * a * b + size_t(dim)];
                        g.esens[size_t(be)] = s;
                    }
                }
        Node<T>& beads = e.arg(*this, 0);
        g.propagate(beads, nullptr);
        for (size_t n = 0; n < g.loc1.size(); ++n) {
            T m = ns[bead_nrot[n]].cur[size_t(bead_res[n]) * bead_nrot[n] + size_t(bead_rot[n])];
            for (int k = 0; k < n_prob_nodes(); ++k) {
                auto& pn = e.arg(*this, 1 + k);
                pn.sens[size_t(g.loc1[n]) * pn.width] += m;
            }
        }
        if (energy) {
            // (calculate_energy_from_marginals, src/rotamer.cpp:915-927)
            T en = 0;
            for (int r : {1, 3, 6})
                for (int i = 0; i < ns[r].n; ++i) en += node_free_energy(ns[r], i);
            for (size_t ix = 0; ix < es[1][1].a.size(); ++ix) en += -std::log(es[1][1].prob[ix]);
            for (auto* E : {&es[3][3], &es[3][6], &es[6][6]})
                for (size_t ix = 0; ix < E->a.size(); ++ix) en += edge_free_energy(*E, int(ix));
            this->pot = en;
        } else {
            this->pot = 0;
        }
    }
    vector<float> value_by_name(const string& w) override {
        if (w == "count_edges_by_type") return HBCoverageNode<T>::count_edges(g);
        if (w == "n_node") return {float(ns[1].n + ns[3].n + ns[6].n)};
        if (w == "read n_bad_solve") return {float(n_bad_solve)};
        if (w == "n_iter") return {float(last_iter)};
        if (w == "node_marginal") {
            // node marginals padded to 6, nodes ordered 1-, 3-, 6-rotamer classes
            vector<float> m;
            for (int r : {1, 3, 6})
                for (int i = 0; i < ns[r].n; ++i)
                    for (int k = 0; k < 6; ++k) m.push_back(k < r ? float(ns[r].cur[size_t(i) * r + size_t(k)]) : 0.f);
            return m;
        }
        if (w == "rotamer_free_energy") {
            // per residue, in residue order (residue_free_energies, src/rotamer.cpp:929-963)
            vector<T> er[7];
            for (int r : {1, 3, 6}) {
                er[r].assign(size_t(ns[r].n), T(0));
                for (int i = 0; i < ns[r].n; ++i) er[r][size_t(i)] += node_free_energy(ns[r], i);
            }
            for (size_t ix = 0; ix < es[1][1].a.size(); ++ix) {
                T en = -std::log(es[1][1].prob[ix]);
                er[1][size_t(es[1][1].a[ix])] += T(0.5) * en;
                er[1][size_t(es[1][1].b[ix])] += T(0.5) * en;
            }
            for (auto* E : {&es[3][3], &es[3][6], &es[6][6]})
                for (size_t ix = 0; ix < E->a.size(); ++ix) {
                    T en = edge_free_energy(*E, int(ix));
                    er[E->r1][size_t(E->a[ix])] += T(0.5) * en;
                    er[E->r2][size_t(E->b[ix])] += T(0.5) * en;
                }
            vector<float> outv;
            std::set<int> seen;
            for (size_t n = 0; n < g.id1.size(); ++n) {
                int id = g.id1[n];
                if ((id & 15) || seen.count(id)) continue;
                seen.insert(id);
                outv.push_back(float(er[(id >> 4) & 15][size_t(id >> 8)]));
            }
            return outv;
        }
        return Node<T>::value_by_name(w);
    }
    vector<float> get_param() override { return vector<float>(g.param.begin(), g.param.end()); }
    void set_param(const vector<float>& p) override {
        if (p.size() != g.param.size()) throw Err("Bad param size");
        g.param.assign(p.begin(), p.end());
        g.update_cutoff();
    }
    vector<float> param_deriv(Engine<T>& e) override { return g.param_deriv(e.arg(*this, 0), nullptr); }
    const vector<std::pair<int, int>>* edges() const override { return &g.edges; }
};

// --------------------------------------------------------------- loading ---
bool is_prefix(const string& p, const string& s) { return s.compare(0, p.size(), p) == 0; }

template <class T> std::unique_ptr<Node<T>> make_node(const string& name, const H5& h) {
    using P = std::unique_ptr<Node<T>>;
    // name-prefix dispatch as the reference registry does (src/deriv_engine.cpp:393-399)
    if (is_prefix("Distance3D", name)) return P(new DistNode<T>(h));
    if (is_prefix("Angle", name)) return P(new AngleNode<T>(h));
    if (is_prefix("Dihedral", name)) return P(new DihedralNode<T>(h));
    if (is_prefix("Spring", name)) return P(new SpringNode<T>(h));
    if (is_prefix("rama_coord", name)) return P(new PasteRamaNode<T>(h));
    if (is_prefix("rama_map_pot", name)) return P(new RamaMapNode<T>(h));
    if (is_prefix("RamaMap2", name)) return P(new RamaMap2Node<T>(h));
    if (is_prefix("Const1D", name)) return P(new ConstNode<T>(h, 1));
    if (is_prefix("Const2D", name)) return P(new ConstNode<T>(h, 2));
    if (is_prefix("Const3D", name)) return P(new ConstNode<T>(h, 3));
    if (is_prefix("cb_membrane_potential", name)) return P(new MembraneCBNode<T>(h));
    if (is_prefix("hb_membrane_potential", name)) return P(new MembraneHBNode<T>(h));
    if (is_prefix("cb_surf_membrane_potential", name)) return P(new MembraneSurfCBNode<T>(h));
    if (is_prefix("hb_surf_membrane_potential", name)) return P(new MembraneSurfHBNode<T>(h));
    if (is_prefix("membranelateral_potential", name)) return P(new LateralNode<T>(h));
    if (is_prefix("surface", name)) return P(new SurfaceNode<T>(h));
    if (is_prefix("SigmoidCoord", name)) return P(new SigmoidCoordNode<T>(h));
    if (is_prefix("SigmoidEnergy", name)) return P(new SigmoidEnergyNode<T>(h, false));
    if (is_prefix("SigmoidLEnergy", name)) return P(new SigmoidEnergyNode<T>(h, true));
    if (is_prefix("Add", name)) return P(new CombineNode<T>(h, CombineNode<T>::ADD));
    if (is_prefix("Mean", name)) return P(new CombineNode<T>(h, CombineNode<T>::MEAN));
    if (is_prefix("Multiply", name)) return P(new CombineNode<T>(h, CombineNode<T>::MUL));
    if (is_prefix("Sum", name)) return P(new SumNode<T>(h));
    if (is_prefix("affine_alignment", name)) return P(new AffineNode<T>(h));
    if (is_prefix("backbone_pairs", name)) return P(new BackbonePairsNode<T>(h));
    if (is_prefix("infer_H_O", name)) return P(new InferHONode<T>(h));
    if (is_prefix("protein_hbond", name)) return P(new ProteinHBondNode<T>(h));
    if (is_prefix("hbond_energy", name)) return P(new HBondEnergyNode<T>(h));
    if (is_prefix("hbond_coverage", name)) return P(new HBCoverageNode<T>(h));
    if (is_prefix("placement_fixed_point_vector_scalar", name)) return P(new PlacementNode<T>(h, "PVS", false));
    if (is_prefix("placement_fixed_point_vector_only", name)) return P(new PlacementNode<T>(h, "PV", false));
    if (is_prefix("placement_fixed_point_only", name)) return P(new PlacementNode<T>(h, "P", false));
    if (is_prefix("placement_fixed_scalar", name)) return P(new PlacementNode<T>(h, "S", false));
    if (is_prefix("placement_scalar", name)) return P(new PlacementNode<T>(h, "S", true));
    if (is_prefix("rotamer", name)) return P(new RotamerNode<T>(h));
    if (is_prefix("weighted_pos", name)) return P(new WeightedPosNode<T>(h));
    if (is_prefix("environment_coverage", name)) return P(new EnvCoverageNode<T>(h));
    if (is_prefix("hb_environment_coverage", name)) return P(new HBEnvCoverageNode<T>(h));
    if (is_prefix("cat_pos", name)) return P(new CatPosNode<T>(h));
    if (is_prefix("sigmoid_coupling", name)) return P(new SigmoidCouplingNode<T>(h));
    if (is_prefix("nonlinear_coupling", name)) return P(new NonlinearCouplingNode<T>(h));
    if (is_prefix("bb_sigmoid_coupling", name)) return P(new BBSigmoidNode<T>(h));
    throw Err("No node type found for name '" + name + "'");
}

template <class T> std::unique_ptr<Engine<T>> build(const string& path, int n_atom) {
    h5lite::File f(path);
    auto e = std::make_unique<Engine<T>>();
    auto pos = std::make_unique<PosNode<T>>();
    pos->name = "pos";
    pos->alloc(n_atom, 3);
    e->index["pos"] = 0;
    e->nodes.push_back(std::move(pos));
    std::map<string, vector<string>> deps;
    for (auto& nm : f.list("/input/potential")) deps[nm] = f.attr_strings("/input/potential/" + nm, "arguments");
    // topological order (src/deriv_engine.cpp:353-426)
    std::set<string> done{"pos"};
    vector<string> order;
    for (size_t round = 0; round <= deps.size(); ++round)
        for (auto& kv : deps) {
            if (done.count(kv.first)) continue;
            bool ok = true;
            for (auto& a : kv.second) ok = ok && done.count(a);
            if (ok) { order.push_back(kv.first); done.insert(kv.first); }
        }
    if (order.size() != deps.size()) throw Err("unsatisfiable dependency in potential graph");
    for (auto& nm : order) {
        H5 h{f, "/input/potential/" + nm};
        std::unique_ptr<Node<T>> node;
        try {
            node = make_node<T>(nm, h);
        } catch (const std::exception& ex) {
            throw Err("while adding '" + nm + "', " + ex.what());
        }
        node->name = nm;
        for (auto& a : deps[nm]) node->args.push_back(e->index.at(a));
        e->index[nm] = int(e->nodes.size());
        e->nodes.push_back(std::move(node));
    }
    return e;
}

// ----------------------------------------------------------------- RNG ---
// Threefry-4x32 with 20 rounds (Salmon et al., SC'11) and the Box-Muller
// normal draws the reference thermostat takes from it (src/random.h:19-67).
inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }
void threefry4x32(const uint32_t ctr[4], const uint32_t key[4], uint32_t out[4]) {
    static const int R[8][2] = {{10, 26}, {11, 21}, {13, 27}, {23, 5}, {6, 20}, {17, 11}, {25, 10}, {18, 20}};
    uint32_t ks[5] = {key[0], key[1], key[2], key[3], 0x1BD11BDAu ^ key[0] ^ key[1] ^ key[2] ^ key[3]};
    uint32_t x[4];
    for (int i = 0; i < 4; ++i) x[i] = ctr[i] + ks[i];
    for (int r = 0; r < 20; ++r) {
        const int* rr = R[r % 8];
        if (r % 2 == 0) {
            x[0] += x[1]; x[1] = rotl32(x[1], rr[0]); x[1] ^= x[0];
            x[2] += x[3]; x[3] = rotl32(x[3], rr[1]); x[3] ^= x[2];
        } else {
            x[0] += x[3]; x[3] = rotl32(x[3], rr[0]); x[3] ^= x[0];
            x[2] += x[1]; x[1] = rotl32(x[1], rr[1]); x[1] ^= x[2];
        }
        if (r % 4 == 3) {
            uint32_t s = uint32_t(r / 4 + 1);
            for (int i = 0; i < 4; ++i) x[i] += ks[(s + uint32_t(i)) % 5];
            x[3] += s;
        }
    }
    for (int i = 0; i < 4; ++i) out[i] = x[i];
}
inline float u01f(uint32_t u) { return float(u) * (1.f / 4294967296.f) + (0.5f / 4294967296.f); }
inline float uneg11f(uint32_t u) { return float(int32_t(u)) * (1.f / 2147483648.f) + (0.5f / 2147483648.f); }
void thermo_normal3(uint32_t seed, uint64_t step, uint32_t atom, float n[3]) {
    uint32_t key[4] = {seed, 0u, 0u, 0u};
    uint32_t ctr[4] = {uint32_t(step & 0xffffffffu), uint32_t(step >> 32), atom, 0u};
    uint32_t b[4];
    threefry4x32(ctr, key, b);
    const float PIf = 3.1415926535897932f;
    float a0 = PIf * uneg11f(b[0]), r0 = std::sqrt(-2.f * std::log(u01f(b[1])));
    float a1 = PIf * uneg11f(b[2]), r1 = std::sqrt(-2.f * std::log(u01f(b[3])));
    n[0] = std::sin(a0) * r0;
    n[1] = std::cos(a0) * r0;
    n[2] = std::sin(a1) * r1;
}

// --------------------------------------------------------------- handles ---
struct Handle {
    int prec = 0;
    int n_atom = 0;
    std::unique_ptr<Engine<float>> ef;
    std::unique_ptr<Engine<double>> ed;
};

template <class T> Engine<T>& eng(Handle* h);
template <> Engine<float>& eng<float>(Handle* h) { return *h->ef; }
template <> Engine<double>& eng<double>(Handle* h) { return *h->ed; }

template <class T> Node<T>& node(Engine<T>& e, const char* name) {
    auto it = e.index.find(name);
    if (it == e.index.end()) throw Err(string("name not found: ") + name);
    return *e.nodes[size_t(it->second)];
}

template <class T> void evaluate_t(Handle* h, const float* pos, double* energy, float* deriv) {
    auto& e = eng<T>(h);
    auto& p = *e.nodes[0];
    for (int i = 0; i < 3 * h->n_atom; ++i) p.out[size_t(i)] = T(pos[i]);
    e.compute(true);
    if (energy) *energy = e.potential;
    if (deriv)
        for (int i = 0; i < 3 * h->n_atom; ++i) deriv[i] = float(p.sens[size_t(i)]);
}

template <class T> void run_t(Handle* h, float* pos, float* mom, int n_round, float dt, float temp, float tau,
                              uint32_t seed, uint64_t round_start) {
    auto& e = eng<T>(h);
    auto& p = *e.nodes[0];
    int n = h->n_atom;
    float delta_t = 3.f * dt;
    float ms = std::exp(-delta_t / tau);
    float nsc = std::sqrt(temp * (1.f - ms * ms));
    vector<T> x(pos, pos + 3 * n), m(mom, mom + 3 * n);
    for (int r = 0; r < n_round; ++r) {
        // thermostat (src/thermostat.cpp:9-18)
        for (int a = 0; a < n; ++a) {
            float z[3];
            thermo_normal3(seed, round_start + uint64_t(r), uint32_t(a), z);
            for (int d = 0; d < 3; ++d) m[3 * size_t(a) + d] = T(ms) * m[3 * size_t(a) + d] + T(nsc) * T(z[d]);
        }
        // integration_cycle (src/deriv_engine.cpp:317-331)
        for (int stage = 0; stage < 3; ++stage) {
            std::copy(x.begin(), x.end(), p.out.begin());
            e.compute(false);
            for (int i = 0; i < 3 * n; ++i) {
                m[size_t(i)] -= T(dt) * p.sens[size_t(i)];
                x[size_t(i)] += T(dt) * m[size_t(i)];
            }
        }
    }
    for (int i = 0; i < 3 * n; ++i) { pos[i] = float(x[size_t(i)]); mom[i] = float(m[size_t(i)]); }
}

#define OCPU_DISPATCH(h, call) ((h)->prec ? call<double> : call<float>)

}  // namespace

extern "C" {

const char* ocpu_last_error(void) { return g_err.c_str(); }

void* ocpu_create(const char* up_path, int n_atom, int precision) {
    try {
        auto h = std::make_unique<Handle>();
        h->prec = precision;
        h->n_atom = n_atom;
        if (precision) h->ed = build<double>(up_path, n_atom);
        else h->ef = build<float>(up_path, n_atom);
        return h.release();
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return nullptr;
    }
}

void ocpu_free(void* h) { delete static_cast<Handle*>(h); }

int ocpu_evaluate(void* hv, const float* pos, double* energy, float* deriv) {
    Handle* h = static_cast<Handle*>(hv);
    try {
        if (h->prec) evaluate_t<double>(h, pos, energy, deriv);
        else evaluate_t<float>(h, pos, energy, deriv);
        return 0;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return 1;
    }
}

#define NODE_CALL(body)                                          \
    Handle* h = static_cast<Handle*>(hv);                        \
    try {                                                        \
        if (h->prec) { auto& N = node(*h->ed, name); auto& E = *h->ed; (void)E; body } \
        else { auto& N = node(*h->ef, name); auto& E = *h->ef; (void)E; body }         \
    } catch (const std::exception& ex) {                         \
        g_err = ex.what();                                       \
        return -1;                                               \
    }

int ocpu_output_dims(void* hv, const char* name, int* n_elem, int* width) {
    NODE_CALL(if (N.potential_node) { *n_elem = 1; *width = 1; } else { *n_elem = N.n_elem; *width = N.width; } return 0;)
}

int ocpu_get_output(void* hv, const char* name, float* out, int n) {
    NODE_CALL(if (N.potential_node) { if (n != 1) return -1; out[0] = float(N.pot); return 0; }
              if (n != int(N.out.size())) return -1;
              for (int i = 0; i < n; ++i) out[i] = float(N.out[size_t(i)]); return 0;)
}

int ocpu_get_sens(void* hv, const char* name, float* out, int n) {
    NODE_CALL(if (N.potential_node) { if (n != 1) return -1; out[0] = float(N.pot); return 0; }
              if (n != int(N.sens.size())) return -1;
              for (int i = 0; i < n; ++i) out[i] = float(N.sens[size_t(i)]); return 0;)
}

int ocpu_value_by_name(void* hv, const char* name, const char* what, float* out, int n) {
    NODE_CALL(auto v = N.value_by_name(what); if (int(v.size()) != n) { g_err = "size " + std::to_string(v.size()); return -1; }
              std::copy(v.begin(), v.end(), out); return 0;)
}

int ocpu_param_size(void* hv, const char* name) { NODE_CALL(return int(N.get_param().size());) }

int ocpu_get_param_deriv(void* hv, const char* name, float* out, int n) {
    NODE_CALL(auto v = N.param_deriv(E); if (int(v.size()) != n) return -1; std::copy(v.begin(), v.end(), out);
              return 0;)
}

int ocpu_set_param(void* hv, const char* name, const float* p, int n) {
    NODE_CALL(N.set_param(std::vector<float>(p, p + n)); return 0;)
}

int ocpu_edges(void* hv, const char* name, int32_t* pairs, int cap) {
    NODE_CALL(auto* ed = N.edges(); if (!ed) return -1; int ne = int(ed->size());
              for (int i = 0; i < ne && i < cap; ++i) { pairs[2 * i] = (*ed)[size_t(i)].first; pairs[2 * i + 1] = (*ed)[size_t(i)].second; }
              return ne;)
}

int ocpu_run(void* hv, float* pos, float* mom, int n_round, float dt, float temperature, float timescale,
             uint32_t seed, uint64_t round_start) {
    Handle* h = static_cast<Handle*>(hv);
    try {
        if (h->prec) run_t<double>(h, pos, mom, n_round, dt, temperature, timescale, seed, round_start);
        else run_t<float>(h, pos, mom, n_round, dt, temperature, timescale, seed, round_start);
        return 0;
    } catch (const std::exception& ex) {
        g_err = ex.what();
        return 1;
    }
}

void ocpu_thermostat_normals(uint32_t seed, uint64_t invocation, int n_atom, float* out) {
    for (int a = 0; a < n_atom; ++a) thermo_normal3(seed, invocation, uint32_t(a), out + 3 * a);
}

}  // extern "C"

extern "C" void ocpu_threefry4x32(const uint32_t* ctr, const uint32_t* key, uint32_t* out) {
    threefry4x32(ctr, key, out);
}
