// llg_diag_host.cpp -- builds the chunked layout of a diagonal observable (llg_diag.h) on the host.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "llg_diag.h"

namespace llg {

namespace {

size_t align16(size_t x) { return (x + 15) & ~(size_t)15; }

template <class T>
T* at(std::vector<unsigned char>& b, size_t off) {
    return reinterpret_cast<T*>(b.data() + off);
}

template <class T>
const T* at(const std::vector<unsigned char>& b, size_t off) {
    return reinterpret_cast<const T*>(b.data() + off);
}

}  // namespace

bool build_diag_obs(int n, int nterms, const int* a, const int* b, const double* c, DiagObsHost& out, std::string& err) {
    if (n < 1 || n > 40) {
        err = "observable: n out of range";
        return false;
    }
    if (nterms < 0 || (nterms > 0 && (!a || !b || !c))) {
        err = "observable: bad term arrays";
        return false;
    }
    for (int k = 0; k < nterms; ++k) {
        if (a[k] < 0 || a[k] >= n || b[k] >= n || b[k] == a[k]) {
            err = "observable: term " + std::to_string(k) + " has a bad qubit";
            return false;
        }
        if (!std::isfinite(c[k])) {
            err = "observable: term " + std::to_string(k) + " has a non-finite coefficient";
            return false;
        }
    }
    DiagObsHost h;
    h.n = n;
    h.nterms = nterms;
    h.L = std::min(n, kDiagMaxLow);
    h.L1 = h.L / 2;
    const int L = h.L;
    std::vector<double> tlo((size_t)1 << L, 0.0);
    std::vector<int32_t> hi_ab;
    std::vector<double> hi_c;
    std::vector<std::vector<std::pair<int32_t, double>>> cross(L);
    for (int k = 0; k < nterms; ++k) {
        int p = a[k], q = b[k] < 0 ? -1 : b[k];
        if (q >= 0 && q < p) std::swap(p, q);  // p < q for pairs; single: q = -1
        const bool p_lo = p < L, q_lo = q < L;  // q = -1 counts as "low" (absent)
        if (q < 0) {
            if (p_lo) {
                for (size_t lo = 0; lo < tlo.size(); ++lo) tlo[lo] += (lo >> p & 1) ? -c[k] : c[k];
            } else {
                hi_ab.push_back(p);
                hi_ab.push_back(-1);
                hi_c.push_back(c[k]);
            }
        } else if (p_lo && q_lo) {
            for (size_t lo = 0; lo < tlo.size(); ++lo) tlo[lo] += ((lo >> p ^ lo >> q) & 1) ? -c[k] : c[k];
        } else if (!p_lo) {
            hi_ab.push_back(p);
            hi_ab.push_back(q);
            hi_c.push_back(c[k]);
        } else {  // p low, q high
            cross[p].push_back({q, c[k]});
        }
    }
    h.n_hi = (int)hi_c.size();
    std::vector<int32_t> cross_off(L + 1, 0), cross_b;
    std::vector<double> cross_c;
    for (int l = 0; l < L; ++l) {
        cross_off[l] = (int32_t)cross_b.size();
        for (auto& t : cross[l]) {
            cross_b.push_back(t.first);
            cross_c.push_back(t.second);
        }
    }
    cross_off[L] = (int32_t)cross_b.size();
    h.n_cross = (int)cross_b.size();
    size_t off = 0;
    h.off_tlo = off;
    off = align16(off + tlo.size() * sizeof(double));
    h.off_hi_ab = off;
    off = align16(off + hi_ab.size() * sizeof(int32_t));
    h.off_hi_c = off;
    off = align16(off + hi_c.size() * sizeof(double));
    h.off_cross_off = off;
    off = align16(off + cross_off.size() * sizeof(int32_t));
    h.off_cross_b = off;
    off = align16(off + cross_b.size() * sizeof(int32_t));
    h.off_cross_c = off;
    off = align16(off + cross_c.size() * sizeof(double));
    h.bytes.assign(std::max<size_t>(off, 16), 0);
    std::memcpy(at<double>(h.bytes, h.off_tlo), tlo.data(), tlo.size() * sizeof(double));
    if (!hi_ab.empty()) std::memcpy(at<int32_t>(h.bytes, h.off_hi_ab), hi_ab.data(), hi_ab.size() * sizeof(int32_t));
    if (!hi_c.empty()) std::memcpy(at<double>(h.bytes, h.off_hi_c), hi_c.data(), hi_c.size() * sizeof(double));
    std::memcpy(at<int32_t>(h.bytes, h.off_cross_off), cross_off.data(), cross_off.size() * sizeof(int32_t));
    if (!cross_b.empty()) std::memcpy(at<int32_t>(h.bytes, h.off_cross_b), cross_b.data(), cross_b.size() * sizeof(int32_t));
    if (!cross_c.empty()) std::memcpy(at<double>(h.bytes, h.off_cross_c), cross_c.data(), cross_c.size() * sizeof(double));
    h.a.assign(a, a + nterms);
    h.b.assign(b, b + nterms);
    h.c.assign(c, c + nterms);
    for (int32_t& v : h.b)
        if (v < 0) v = -1;
    out = std::move(h);
    return true;
}

bool diag_obs_same(const DiagObsHost& h, int n, int nterms, const int* a, const int* b, const double* c) {
    if (h.bytes.empty() || h.n != n || h.nterms != nterms) return false;
    for (int k = 0; k < nterms; ++k)
        if (h.a[k] != a[k] || h.b[k] != (b[k] < 0 ? -1 : b[k]) || !(h.c[k] == c[k])) return false;
    return true;
}

DiagObs diag_obs_view(const DiagObsHost& h, const void* dev) {
    DiagObs v;
    std::memset(&v, 0, sizeof(v));
    const unsigned char* base = static_cast<const unsigned char*>(dev);
    v.n = h.n;
    v.L = h.L;
    v.L1 = h.L1;
    v.n_hi = h.n_hi;
    v.n_cross = h.n_cross;
    v.t_lo = reinterpret_cast<const double*>(base + h.off_tlo);
    v.hi_ab = reinterpret_cast<const int32_t*>(base + h.off_hi_ab);
    v.hi_c = reinterpret_cast<const double*>(base + h.off_hi_c);
    v.cross_off = reinterpret_cast<const int32_t*>(base + h.off_cross_off);
    v.cross_b = reinterpret_cast<const int32_t*>(base + h.off_cross_b);
    v.cross_c = reinterpret_cast<const double*>(base + h.off_cross_c);
    v.diag = nullptr;
    return v;
}

void diag_obs_eval_host(const DiagObsHost& h, double* out) {
    const int L = h.L, L1 = h.L1, L2 = L - L1;
    const double* tlo = at<double>(h.bytes, h.off_tlo);
    const int32_t* hi_ab = at<int32_t>(h.bytes, h.off_hi_ab);
    const double* hi_c = at<double>(h.bytes, h.off_hi_c);
    const int32_t* coff = at<int32_t>(h.bytes, h.off_cross_off);
    const int32_t* cb = at<int32_t>(h.bytes, h.off_cross_b);
    const double* cc = at<double>(h.bytes, h.off_cross_c);
    const uint64_t nchunks = 1ULL << (h.n - L);
    std::vector<double> heff(L), h1((size_t)1 << L1), h2((size_t)1 << L2);
    for (uint64_t ch = 0; ch < nchunks; ++ch) {
        const uint64_t hi = ch << L;
        double dhi = 0.0;
        for (int k = 0; k < h.n_hi; ++k) {
            int par = (int)(hi >> hi_ab[2 * k] & 1);
            if (hi_ab[2 * k + 1] >= 0) par ^= (int)(hi >> hi_ab[2 * k + 1] & 1);
            dhi += par ? -hi_c[k] : hi_c[k];
        }
        for (int l = 0; l < L; ++l) {
            double v = 0.0;
            for (int k = coff[l]; k < coff[l + 1]; ++k) v += (hi >> cb[k] & 1) ? -cc[k] : cc[k];
            heff[l] = v;
        }
        for (size_t j = 0; j < h1.size(); ++j) {
            double v = 0.0;
            for (int l = 0; l < L1; ++l) v += (j >> l & 1) ? -heff[l] : heff[l];
            h1[j] = v;
        }
        for (size_t j = 0; j < h2.size(); ++j) {
            double v = 0.0;
            for (int l = 0; l < L2; ++l) v += (j >> l & 1) ? -heff[L1 + l] : heff[L1 + l];
            h2[j] = v;
        }
        for (uint64_t lo = 0; lo < (1ULL << L); ++lo)
            out[hi | lo] = ((tlo[lo] + h1[lo & (h1.size() - 1)]) + h2[lo >> L1]) + dhi;
    }
}

}  // namespace llg
