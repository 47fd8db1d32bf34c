// lattice.cpp -- CObjects lattice -> device element stream.
//
// Per-element constants that the reference computes on every call are folded
// here, with the reference's own operation order so results stay
// bit-identical: the cavity's DEG2RAD*lag and (2*pi/c)*frequency
// (be_cavity/track.h:46-55), the XYShift's negated offsets
// (be_xyshift/track.h:45-46).  Slice arrays of BeamBeam6D, addressed by
// relative offsets in the reference (be_beamfields.h:23-27), are laid out
// contiguously after the fixed part.
#include "lattice.h"

#include <algorithm>
#include <array>
#include <cmath>
#include <map>

namespace stg {

namespace {

constexpr double kPi = 3.1415926535897932384626433832795028841971693993751;
constexpr double kClight = 299792458.0;
constexpr double kEps0 = 8.854187817620e-12;

struct Emitter {
    std::vector<uint64_t> recs;     // records, unchunked
    std::vector<uint64_t> rec_len;  // per record
    // {record, parameter index, offset in the side data}: parameter words
    // that receive the device address of out-of-line data
    std::vector<std::array<uint64_t, 3>> side_refs;
    // the same for offsets into the device-only region after the side data
    std::vector<std::array<uint64_t, 3>> device_refs;
    void push(uint32_t op, uint32_t aux, const std::vector<uint64_t> &params)
    {
        uint32_t const n = (uint32_t)params.size() + 1;
        recs.push_back(make_header(op, n, aux));
        recs.insert(recs.end(), params.begin(), params.end());
        rec_len.push_back(n);
    }
};

bool bad(std::string *err, uint64_t i, const char *what)
{
    if (err) *err = "element " + std::to_string(i) + ": " + what;
    return false;
}

// Opcode of an element whose map is skipped or disabled by its feature flag.
uint32_t flagged_op(int flag) { return flag == MAP_SKIP ? OP_NOP : OP_FAIL; }

// Cell tables of one lattice are capped at this many cells in total
// (64 coefficients, 512 bytes each: 32 GiB).
constexpr uint64_t kMaxTricubCells = (uint64_t)1 << 26;

}  // namespace

bool compile_lattice(const ImageView &img, uint64_t begin, uint64_t end,
                     const CompileOptions &opt, CompiledStream *out, std::string *err)
{
    if (begin > end || end > img.num_objects) return bad(err, end, "line range outside the lattice");
    Emitter em;
    out->monitor_elements.clear();
    out->side.clear();
    out->side_fixups.clear();
    out->side_device_words = 0;
    out->tricub_tables.clear();
    std::map<uint64_t, size_t> tricub_of_data;  // TriCubData address -> table
    uint64_t tricub_cells = 0;
    out->s_table.assign(1, 0.0);
    uint32_t op_mask = 0;
    for (uint64_t i = begin; i < end; ++i) {
        uint64_t const t = img.type_of(i);
        uint64_t const nw = img.size_bytes(i) / 8;
        const uint64_t *w = img.words(i);
        auto need = [&](uint64_t k) { return nw >= k; };
        auto d = [&](uint64_t k) { return w[k]; };
        std::vector<uint64_t> p;
        uint32_t op = OP_FAIL_LOST, aux = 0;
        switch (t) {
        case ST_OBJECT_TYPE_DRIFT:
        case ST_OBJECT_TYPE_DRIFT_EXACT: {
            if (!need(1)) return bad(err, i, "truncated drift");
            double const L = w2d(w[0]);
            op = (t == ST_OBJECT_TYPE_DRIFT) ? OP_DRIFT : OP_DRIFT_EXACT;
            bool const ap = opt.aperture_mode == 2 ||
                            (opt.aperture_mode == 1 && L >= opt.aperture_min_length);
            aux = ap ? DRIFT_APERTURE : 0u;
            p = {d(0)};
            break;
        }
        case ST_OBJECT_TYPE_MULTIPOLE: {
            if (!need(5)) return bad(err, i, "truncated multipole");
            int64_t const order = (int64_t)w[0];
            if (order < 0 || order > 64) return bad(err, i, "multipole order out of range");
            const uint64_t *bal = img.deref(i, 4);
            if (!bal) return bad(err, i, "multipole bal pointer outside the buffer");
            double const hxl = w2d(w[2]), hyl = w2d(w[3]);
            bool const curv = (hxl > 0.0) || (hyl > 0.0) || (hxl < 0.0) || (hyl < 0.0);
            op = curv ? OP_MULTIPOLE_CURV : OP_MULTIPOLE;
            aux = (uint32_t)order;
            p.assign(bal, bal + 2 * order + 2);
            if (curv) {
                double const length = w2d(w[1]);
                p.push_back(w[2]);
                p.push_back(w[3]);
                p.push_back(w[1]);
                // hxl / length, hyl / length (0 without length): the
                // derivative kernels' form of the b1 / a1 terms
                p.push_back(d2w(length > 0.0 ? hxl / length : 0.0));
                p.push_back(d2w(length > 0.0 ? hyl / length : 0.0));
            }
            break;
        }
        case ST_OBJECT_TYPE_CAVITY: {
            if (!need(3)) return bad(err, i, "truncated cavity");
            double const DEG2RAD = kPi / 180.0;
            double const K_FACTOR = (2.0 * kPi) / kClight;
            op = OP_CAVITY;
            p = {w[0], d2w(K_FACTOR * w2d(w[1])), d2w(DEG2RAD * w2d(w[2]))};
            break;
        }
        case ST_OBJECT_TYPE_XYSHIFT:
            if (!need(2)) return bad(err, i, "truncated xyshift");
            op = OP_XYSHIFT;
            p = {d2w(-(w2d(w[0]))), d2w(-(w2d(w[1])))};
            break;
        case ST_OBJECT_TYPE_SROTATION:
            if (!need(2)) return bad(err, i, "truncated srotation");
            op = OP_SROTATION;
            p = {w[0], w[1]};
            break;
        case ST_OBJECT_TYPE_LIMIT_RECT:
            if (!need(4)) return bad(err, i, "truncated limit_rect");
            op = OP_LIMIT_RECT;
            p.assign(w, w + 4);
            break;
        case ST_OBJECT_TYPE_LIMIT_ELLIPSE:
            if (!need(3)) return bad(err, i, "truncated limit_ellipse");
            op = OP_LIMIT_ELLIPSE;
            p.assign(w, w + 3);
            // the kernel compares t = x^2 b^2 + y^2 a^2 <= a^2 b^2 as integers
            // when all three are non-negative (then t >= +0 or NaN)
            if (std::signbit(w2d(w[0])) || std::signbit(w2d(w[1])) || std::signbit(w2d(w[2])) ||
                std::isnan(w2d(w[2])))
                aux = 1u;
            break;
        case ST_OBJECT_TYPE_LIMIT_RECT_ELLIPSE:
            if (!need(5)) return bad(err, i, "truncated limit_rect_ellipse");
            op = OP_LIMIT_RECT_ELLIPSE;
            p.assign(w, w + 5);
            break;
        case ST_OBJECT_TYPE_DIPEDGE:
            if (!need(2)) return bad(err, i, "truncated dipedge");
            op = OP_DIPEDGE;
            p.assign(w, w + 2);
            break;
        case ST_OBJECT_TYPE_RF_MULTIPOLE: {
            if (!need(6)) return bad(err, i, "truncated rf multipole");
            int64_t const order = (int64_t)w[0];
            if (order < 0 || order > 64) return bad(err, i, "rf multipole order out of range");
            const uint64_t *bal = img.deref(i, 4);
            const uint64_t *ph = img.deref(i, 5);
            if (!bal || !ph) return bad(err, i, "rf multipole pointer outside the buffer");
            op = OP_RF_MULTIPOLE;
            aux = (uint32_t)order;
            p = {w[1], w[2], w[3]};
            p.insert(p.end(), bal, bal + 2 * order + 2);
            p.insert(p.end(), ph, ph + 2 * order + 2);
            break;
        }
        case ST_OBJECT_TYPE_BEAM_BEAM_4D: {
            if (opt.track_bb4d != MAP_ENABLED) {
                op = flagged_op(opt.track_bb4d);
                break;
            }
            if (!need(2)) return bad(err, i, "truncated beam-beam 4d");
            const uint64_t *bd = img.deref(i, 1);
            if (!bd || w[0] < 11) return bad(err, i, "beam-beam 4d data missing");
            if (!(w2d(bd[10]) > 0.)) {
                op = OP_NOP;
            } else {
                op = OP_BB4D;
                p.assign(bd, bd + 11);
            }
            break;
        }
        case ST_OBJECT_TYPE_BEAM_BEAM_6D: {
            if (opt.track_bb6d != MAP_ENABLED) {
                op = flagged_op(opt.track_bb6d);
                break;
            }
            if (!need(2)) return bad(err, i, "truncated beam-beam 6d");
            const uint64_t *bd = img.deref(i, 1);
            if (!bd || w[0] < 38) return bad(err, i, "beam-beam 6d data missing");
            if (!(w2d(bd[33]) > 0.)) {
                op = OP_NOP;
                break;
            }
            int64_t const ns = (int64_t)(int)(int64_t)bd[18];
            if (ns < 0 || ns > 100000) return bad(err, i, "beam-beam 6d slice count out of range");
            op = OP_BB6D;
            aux = (uint32_t)ns;
            {
                auto f = [&](int k) { return w2d(bd[k]); };  // Sigma at words 6-15
                bool finite = true;
                for (int k = 6; k < 18; ++k) finite = finite && std::isfinite(f(k));
                if (finite && f(6) == f(13) && f(7) == f(14) && f(10) == f(15) && f(8) == 0.0 &&
                    f(9) == 0.0 && f(11) == 0.0 && f(12) == 0.0 && f(16) > 0.0 && f(17) > 0.0)
                    aux |= BB6D_ROUND;
            }
            p.assign(bd, bd + 34);
            for (int f = 34; f < 38; ++f) {
                uint64_t const off = (uint64_t)f + bd[f] + 1;
                if (off + (uint64_t)ns > w[0]) return bad(err, i, "beam-beam 6d slice array outside data");
                p.insert(p.end(), bd + off, bd + off + ns);
            }
            break;
        }
        case ST_OBJECT_TYPE_SC_COASTING:
            if (opt.track_sc != MAP_ENABLED) {
                op = flagged_op(opt.track_sc);
                break;
            }
            if (!need(9)) return bad(err, i, "truncated space-charge coasting");
            op = OP_SC_COASTING;
            p.assign(w, w + 9);
            break;
        case ST_OBJECT_TYPE_SC_QGAUSSIAN_PROF:
            if (opt.track_sc != MAP_ENABLED) {
                op = flagged_op(opt.track_sc);
                break;
            }
            if (!need(11)) return bad(err, i, "truncated space-charge q-gaussian");
            op = OP_SC_QGAUSS;
            p.assign(w, w + 11);
            {
                // element constants of the kick, as track.h:203-268 and
                // NS(Math_q_gauss) compute them for every particle
                double const sqrt_beta = 1.0 / (std::sqrt(2.0) * w2d(w[1]));
                double const omq = 1.0 - w2d(w[8]);
                double const abs_omq = (omq >= 0.0) ? omq : -omq;
                for (double v : {sqrt_beta, sqrt_beta * sqrt_beta, sqrt_beta / w2d(w[9]),
                                 abs_omq >= 1e-6 ? 1.0 / omq : 0.0})
                    p.push_back(d2w(v));
                // the round field's constants (gauss_fields.h:138-148), used
                // by the fast arithmetic policy in place of two divisions
                double const sx = w2d(w[2]), sy = w2d(w[3]), msd = w2d(w[7]);
                double const sigma = 0.5 * (sx + sy);
                bool const round = std::fabs(sx - sy) < msd;
                p.push_back(d2w(round ? 0.5 / (sigma * sigma) : 0.0));
                p.push_back(d2w(round ? 1.0 / (2.0 * kPi * kEps0 * sigma) : 0.0));
                if (round) aux |= SC_ROUND;
                // the elliptic field's constants (gauss_fields.h:150-190)
                bool const ell = !round && sx != sy && sx > 0.0 && sy > 0.0;
                double const S = ell ? std::sqrt(2.0 * std::fabs(sx * sx - sy * sy)) : 0.0;
                double const kSqrtPi = 1.7724538509055160272981674833411451827975494561224;
                for (double v : {ell ? 1.0 / S : 0.0, ell ? 1.0 / (2.0 * kEps0 * kSqrtPi * S) : 0.0,
                                 ell ? sy / sx : 0.0, ell ? sx / sy : 0.0,
                                 ell ? 1.0 / (2.0 * sx * sx) : 0.0,
                                 ell ? 1.0 / (2.0 * sy * sy) : 0.0})
                    p.push_back(d2w(v));
                if (ell) aux |= (sx > sy) ? SC_ELL_X : SC_ELL_Y;
                // the fast policy's round Gaussian kick in one factor:
                // length N sqrt_beta / cq / (2 pi eps0), and 1 / sigma for
                // the kick near the axis
                if (abs_omq < 1e-6) aux |= SC_Q1;
                p.push_back(d2w(round ? w2d(w[4]) * w2d(w[0]) * (sqrt_beta / w2d(w[9])) *
                                            (1.0 / (2.0 * kPi * kEps0))
                                      : 0.0));
                p.push_back(d2w(round ? 1.0 / sigma : 0.0));
            }
            break;
        case ST_OBJECT_TYPE_SC_INTERPOLATED_PROF: {
            // With space charge skipped or disabled the reference's
            // dispatcher has no case label for this type: the preprocessor
            // branch that starts in the q-Gaussian case (track.h:537-575)
            // encloses it, so the default branch loses the particle.
            if (opt.track_sc != MAP_ENABLED) break;
            // be_beamfields/track.h:273-337.  interpol_data_addr (field 6)
            // is a plain address of a NS(LineDensityProfileData): inside
            // this buffer, or else a host address, which the reference's CPU
            // tracking dereferences as it is (the data is copied into the
            // compiled record here); 0 selects the fallback density.
            if (!need(10)) return bad(err, i, "truncated interpolated space charge");
            op = OP_SC_INTERP;
            // N, sigma_x, sigma_y, length, x_co, y_co, fallback, min_sigma_diff
            p = {w[0], w[1], w[2], w[3], w[4], w[5], w[7], w[8]};
            uint64_t method = 255, nv = 0, z0 = 0, dz = 0, voff = 0, doff = 0;
            std::vector<uint64_t> data;
            if (w[6] != 0) {
                uint64_t const dw = img.word_of(w[6]);
                bool const inside = dw != UINT64_MAX && dw + 7 <= img.size_words;
                const uint64_t *ld =
                    inside ? img.img + dw : reinterpret_cast<const uint64_t *>((uintptr_t)w[6]);
                int64_t const cap = (int64_t)ld[1];
                if (ld[0] != 255u && (int64_t)ld[6] > 0) {
                    if (cap <= 0 || cap > (int64_t)1 << 20 || ld[2] == 0 || ld[3] == 0)
                        return bad(err, i, "line-density data without arrays");
                    // the window the interpolation reads: from the first
                    // array's start to the end of the second (the
                    // reference's y[idx + 1] in the last interval reads the
                    // first derivative); reads outside it give 0
                    uint64_t const va = ld[2], da = ld[3];
                    uint64_t const lo = std::min(va, da);
                    uint64_t const hi = std::max(va, da) + (uint64_t)cap * 8u;
                    if ((hi - lo) / 8u > ((uint64_t)1 << 21))
                        return bad(err, i, "line-density arrays too far apart");
                    if (inside) {
                        uint64_t const lw = img.word_of(lo);
                        uint64_t const hw = img.word_of(hi - 8u);
                        if (lw == UINT64_MAX || hw == UINT64_MAX)
                            return bad(err, i, "line-density arrays outside the lattice buffer");
                        data.assign(img.img + lw, img.img + hw + 1);
                    } else {
                        const uint64_t *src = reinterpret_cast<const uint64_t *>((uintptr_t)lo);
                        data.assign(src, src + (hi - lo) / 8u);
                    }
                    voff = (va - lo) / 8u;
                    doff = (da - lo) / 8u;
                    method = ld[0];
                    nv = ld[6];
                    z0 = ld[4];
                    dz = ld[5];
                }
            }
            aux = (method != 255u && nv > 0) ? 1u : 0u;
            // the table stays in global memory (read through L2), its
            // address in the last parameter word
            p.insert(p.end(), {method, nv, z0, dz, voff, doff, (uint64_t)data.size(), 0});
            em.side_refs.push_back({(uint64_t)em.rec_len.size(), (uint64_t)p.size() - 1,
                                    (uint64_t)out->side.size()});
            out->side.insert(out->side.end(), data.begin(), data.end());
            out->side.resize((out->side.size() + 1) & ~(size_t)1);  // 16-byte aligned tables
            break;
        }
        case ST_OBJECT_TYPE_BEAM_MONITOR: {
            if (!need(8)) return bad(err, i, "truncated beam monitor");
            op = OP_MONITOR;
            uint64_t optr = 0;
            int64_t ocap = 0;
            if (opt.monitor_output) {
                auto o = opt.monitor_output(i);
                optr = o.first;
                ocap = o.second;
            }
            if ((int64_t)w[2] <= 0 || (int64_t)w[0] <= 0) optr = 0;  // skip/num_stores must be > 0
            p = {w[0], w[1], w[2], w[4], w[5], w[6], w[7], optr, (uint64_t)ocap};
            out->monitor_elements.push_back(i);
            break;
        }
        case ST_OBJECT_TYPE_TRICUB_DATA:
            // track.h:446-460: skipped unless the TriCub map is disabled
            op = opt.track_tricub == MAP_DISABLED ? OP_FAIL : OP_NOP;
            break;
        case ST_OBJECT_TYPE_TRICUB: {
            // TriCub is "disabled" in the reference's default build
            // (Settings.cmake.default): tracking returns failure.
            if (opt.track_tricub != MAP_ENABLED) {
                op = flagged_op(opt.track_tricub);
                break;
            }
            // be_tricub/track.h:51-224.  data_addr (field 7) is a plain
            // address of a NS(TriCubData) {x0, dx, nx, y0, dy, ny, z0, dz,
            // nz, mirror_x, mirror_y, mirror_z, table_addr}
            // (be_tricub.h:33-52): inside this buffer, or else a host
            // address (a stored buffer the job assigned it from).
            if (!need(8)) return bad(err, i, "truncated tricub");
            uint64_t const addr = w[7];
            uint64_t const dw = addr ? img.word_of(addr) : UINT64_MAX;
            bool const inside = dw != UINT64_MAX && dw + 13 <= img.size_words;
            if (addr == 0) {
                op = OP_FAIL;  // no data: the reference dereferences null
                break;
            }
            const uint64_t *td = inside ? img.img + dw : reinterpret_cast<const uint64_t *>((uintptr_t)addr);
            int64_t const nx = (int64_t)td[2], ny = (int64_t)td[5], nz = (int64_t)td[8];
            if (nx < 2 || ny < 2 || nz < 2) {
                op = OP_FAIL;  // no grid cell: every particle is outside
                break;
            }
            uint64_t const cells = (uint64_t)(nx - 1) * (uint64_t)(ny - 1) * (uint64_t)(nz - 1);
            if (nx > ((int64_t)1 << 26) || ny > ((int64_t)1 << 26) || nz > ((int64_t)1 << 26) ||
                cells > kMaxTricubCells)
                return bad(err, i, "tricub grid too large");
            auto found = tricub_of_data.find(addr);
            size_t tab;
            if (found != tricub_of_data.end()) {
                tab = found->second;
            } else {
                if (tricub_cells + cells > kMaxTricubCells)
                    return bad(err, i, "tricub grids too large in total");
                uint64_t const nvals = (uint64_t)nx * (uint64_t)ny * (uint64_t)nz * 8u;
                const uint64_t *nodes;
                if (inside) {
                    uint64_t const tw = img.word_of(td[12]);
                    if (tw == UINT64_MAX || tw + nvals > img.size_words)
                        return bad(err, i, "tricub table outside the lattice buffer");
                    nodes = img.img + tw;
                } else {
                    nodes = reinterpret_cast<const uint64_t *>((uintptr_t)td[12]);
                    if (!nodes) return bad(err, i, "tricub data without a table");
                }
                CompiledStream::TricubTable t;
                t.nodes = out->side.size();
                t.cells = out->side_device_words;
                t.nx = nx;
                t.ny = ny;
                t.nz = nz;
                out->side.insert(out->side.end(), nodes, nodes + nvals);
                out->side.resize((out->side.size() + 1) & ~(size_t)1);
                out->side_device_words += cells * 64u;
                tricub_cells += cells;
                tab = out->tricub_tables.size();
                out->tricub_tables.push_back(t);
                tricub_of_data[addr] = tab;
            }
            op = OP_TRICUB;
            double const dx = w2d(td[1]), dy = w2d(td[4]), dz = w2d(td[7]);
            double const inv_dx = 1. / dx, inv_dy = 1. / dy, inv_dz = 1. / dz;
            double const length = w2d(w[6]);
            aux = ((int64_t)td[9] == 1 ? TRICUB_MIRROR_X : 0u) |
                  ((int64_t)td[10] == 1 ? TRICUB_MIRROR_Y : 0u) |
                  ((int64_t)td[11] == 1 ? TRICUB_MIRROR_Z : 0u);
            p = {w[0], w[1], w[2], w[3], w[4], w[5],
                 d2w(length * inv_dx), d2w(length * inv_dy), d2w(length * inv_dz),
                 td[0], td[3], td[6],
                 d2w(inv_dx), d2w(inv_dy), d2w(inv_dz),
                 d2w((double)(nx - 2)), d2w((double)(ny - 2)), d2w((double)(nz - 2)),
                 (uint64_t)(nx - 1), (uint64_t)(ny - 1), 0};
            em.device_refs.push_back({(uint64_t)em.rec_len.size(), (uint64_t)p.size() - 1,
                                      out->tricub_tables[tab].cells});
            break;
        }
        default:
            op = OP_FAIL_LOST;
            break;
        }
        op_mask |= 1u << op;
        em.push(op, aux, p);
        double s_next = out->s_table.back();
        if (t == ST_OBJECT_TYPE_DRIFT || t == ST_OBJECT_TYPE_DRIFT_EXACT) s_next += w2d(w[0]);
        out->s_table.push_back(s_next);
    }
    // chunking
    uint64_t maxrec = 1;
    for (uint64_t n : em.rec_len) maxrec = std::max<uint64_t>(maxrec, n);
    uint64_t cw = (uint64_t)std::max<int32_t>(opt.min_chunk_words, 64);
    while (cw < maxrec + 1) cw *= 2;
    cw = (cw + 1) & ~(uint64_t)1;
    out->words.clear();
    out->words.reserve(em.recs.size() + em.rec_len.size() + cw);
    uint64_t used = 0, pos = 0;
    int32_t nchunks = 0;
    auto close_chunk = [&]() {
        out->words.push_back(make_header(OP_END, 1, 0));
        ++used;
        while (used < cw) {
            out->words.push_back(0);
            ++used;
        }
        ++nchunks;
        used = 0;
    };
    out->elem_offset.clear();
    out->elem_offset.reserve(em.rec_len.size());
    for (uint64_t r = 0; r < em.rec_len.size(); ++r) {
        uint64_t const n = em.rec_len[r];
        if (used + n + 1 > cw) close_chunk();
        out->elem_offset.push_back((int64_t)out->words.size());
        out->words.insert(out->words.end(), em.recs.begin() + pos, em.recs.begin() + pos + n);
        used += n;
        pos += n;
    }
    if (used > 0 || nchunks == 0) close_chunk();
    for (const auto &r : em.side_refs)
        out->side_fixups.push_back({(uint64_t)out->elem_offset[r[0]] + 1u + r[1], r[2]});
    // the device-only region follows the side data (kept 16-byte aligned)
    uint64_t const device_at = out->side.size();
    for (auto &t : out->tricub_tables) t.cells += device_at;
    for (const auto &r : em.device_refs)
        out->side_fixups.push_back({(uint64_t)out->elem_offset[r[0]] + 1u + r[1], device_at + r[2]});
    out->info.num_elements = (int64_t)(end - begin);
    out->info.num_chunks = nchunks;
    out->info.chunk_words = (int32_t)cw;
    out->info.max_record_words = (int32_t)maxrec;
    out->info.num_monitors = (int32_t)out->monitor_elements.size();
    out->info.op_mask = op_mask;
    return true;
}

}  // namespace stg
