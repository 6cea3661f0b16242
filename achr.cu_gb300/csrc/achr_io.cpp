// Host input/output of the ACHRCuda drop-in: fixed-MPS reader, warmup CSV
// reader and the File<ii> writer.  Replaces the reference's GLPK model read
// (ACHRcu/ACHRCuda.cu:560-597), its strtok/atof CSV parsing (:387-412,
// :675-689) and its fprintf("%f") output loop (:744-756).
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/achr.h"

// The C ABI's achr_last_error() lives in the CUDA translation unit; I/O
// errors are routed there through this hook.
extern "C" void achr_io_set_error(const char *msg);

namespace {

achr_status io_fail(achr_status st, const std::string &msg) {
    achr_io_set_error(msg.c_str());
    return st;
}

bool read_file(const char *path, std::string &data) {
    FILE *f = std::fopen(path, "rb");
    if (!f) return false;
    std::fseek(f, 0, SEEK_END);
    long len = std::ftell(f);
    std::fseek(f, 0, SEEK_SET);
    if (len < 0) {
        std::fclose(f);
        return false;
    }
    data.resize((size_t)len);
    size_t got = len ? std::fread(&data[0], 1, (size_t)len, f) : 0;
    std::fclose(f);
    return got == (size_t)len;
}

void split_ws(const std::string &line, std::vector<std::string> &tok) {
    tok.clear();
    size_t i = 0, n = line.size();
    while (i < n) {
        while (i < n && (line[i] == ' ' || line[i] == '\t' || line[i] == '\r')) ++i;
        if (i >= n) break;
        size_t j = i;
        while (j < n && line[j] != ' ' && line[j] != '\t' && line[j] != '\r') ++j;
        tok.emplace_back(line.substr(i, j - i));
        i = j;
    }
}

bool parse_double(const std::string &s, double &v) {
    if (s.empty()) return false;
    char *end = nullptr;
    errno = 0;
    v = std::strtod(s.c_str(), &end);
    return end && *end == '\0';
}

}  // namespace

extern "C" {

void achr_free(void *p) { std::free(p); }

void achr_free_model(achr_model_buf *m) {
    if (!m) return;
    std::free(m->row_buf);
    std::free(m->col_buf);
    std::free(m->val_buf);
    std::free(m->lb_buf);
    std::free(m->ub_buf);
    std::memset(m, 0, sizeof(*m));
}

achr_status achr_read_mps(const char *path, achr_model_buf *out) {
    if (!path || !out) return io_fail(ACHR_ERR_INVALID, "NULL argument");
    std::memset(out, 0, sizeof(*out));
    std::string data;
    if (!read_file(path, data)) return io_fail(ACHR_ERR_IO, std::string("cannot read MPS file ") + path);

    enum Sec { NONE, NAME, ROWS, COLUMNS, RHS, RANGES, BOUNDS, OTHER, END } sec = NONE;
    std::unordered_map<std::string, int> row_of, col_of;
    std::string obj_row;
    std::vector<int32_t> rows, cols;
    std::vector<double> vals, lb, ub;
    std::vector<std::string> tok;
    int nrows = 0;
    size_t pos = 0, lineno = 0;
    const double inf = std::numeric_limits<double>::infinity();
    while (pos < data.size() && sec != END) {
        size_t eol = data.find('\n', pos);
        if (eol == std::string::npos) eol = data.size();
        std::string line = data.substr(pos, eol - pos);
        pos = eol + 1;
        ++lineno;
        if (line.empty() || line[0] == '*') continue;
        split_ws(line, tok);
        if (tok.empty()) continue;
        auto bad = [&](const std::string &why) {
            return io_fail(ACHR_ERR_PARSE, std::string(path) + ":" + std::to_string(lineno) + ": " + why);
        };
        if (line[0] != ' ' && line[0] != '\t') {  // section header in column 1
            const std::string &h = tok[0];
            if (h == "NAME") sec = NAME;
            else if (h == "ROWS") sec = ROWS;
            else if (h == "COLUMNS") sec = COLUMNS;
            else if (h == "RHS") sec = RHS;
            else if (h == "RANGES") sec = RANGES;
            else if (h == "BOUNDS") sec = BOUNDS;
            else if (h == "ENDATA") sec = END;
            else if (h == "OBJSENSE" || h == "OBJSENCE" || h == "OBJNAME") sec = OTHER;
            else return bad("unknown section '" + h + "'");
            continue;
        }
        switch (sec) {
            case ROWS: {
                if (tok.size() < 2) return bad("ROWS entry needs a type and a name");
                const std::string &t = tok[0], &name = tok[1];
                if (t != "N" && t != "E" && t != "L" && t != "G") return bad("unknown row type '" + t + "'");
                if (row_of.count(name) || name == obj_row) return bad("duplicate row '" + name + "'");
                if (t == "N" && obj_row.empty()) {
                    obj_row = name;  // the objective: not a row of S
                } else {
                    row_of[name] = nrows++;  // further free rows are kept as rows of S
                }
                break;
            }
            case COLUMNS: {
                if (line.find("'MARKER'") != std::string::npos) break;
                if (tok.size() != 3 && tok.size() != 5) return bad("COLUMNS entry needs 3 or 5 fields");
                const std::string &cname = tok[0];
                auto it = col_of.find(cname);
                int c;
                if (it == col_of.end()) {
                    c = (int)lb.size();
                    col_of[cname] = c;
                    lb.push_back(0.0);
                    ub.push_back(inf);
                } else {
                    c = it->second;
                }
                for (size_t f = 1; f + 1 < tok.size(); f += 2) {
                    double v;
                    if (!parse_double(tok[f + 1], v)) return bad("bad coefficient '" + tok[f + 1] + "'");
                    if (tok[f] == obj_row) continue;
                    auto r = row_of.find(tok[f]);
                    if (r == row_of.end()) return bad("unknown row '" + tok[f] + "'");
                    rows.push_back(r->second);
                    cols.push_back(c);
                    vals.push_back(v);
                }
                break;
            }
            case BOUNDS: {
                const std::string &t = tok[0];
                const bool has_value = !(t == "FR" || t == "MI" || t == "PL" || t == "BV");
                // [type, set, column, value] or, with the set name left blank, [type, column, value]
                std::string cname;
                double v = 0.0;
                if (has_value) {
                    if (tok.size() == 4) cname = tok[2];
                    else if (tok.size() == 3) cname = tok[1];
                    else return bad("bound entry needs a column and a value");
                    if (!parse_double(tok.back(), v)) return bad("bad bound value '" + tok.back() + "'");
                } else {
                    if (tok.size() == 3) cname = tok[2];
                    else if (tok.size() == 2) cname = tok[1];
                    else return bad("bound entry needs a column");
                }
                auto it = col_of.find(cname);
                if (it == col_of.end()) return bad("bound on unknown column '" + cname + "'");
                const int c = it->second;
                if (t == "UP") {
                    ub[c] = v;
                    if (v < 0.0 && lb[c] == 0.0) lb[c] = -inf;  // classic MPS rule for a negative UP bound
                } else if (t == "LO") lb[c] = v;
                else if (t == "FX") lb[c] = ub[c] = v;
                else if (t == "FR") { lb[c] = -inf; ub[c] = inf; }
                else if (t == "MI") lb[c] = -inf;
                else if (t == "PL") ub[c] = inf;
                else if (t == "BV") { lb[c] = 0.0; ub[c] = 1.0; }
                else if (t == "LI") lb[c] = v;
                else if (t == "UI") ub[c] = v;
                else if (t == "SC") ub[c] = v;
                else return bad("unknown bound type '" + t + "'");
                break;
            }
            case NAME:
            case RHS:
            case RANGES:
            case OTHER:
                break;  // RHS, RANGES and the objective sense are not used by the sampler
            case NONE:
                return bad("data line before any section");
            case END:
                break;
        }
    }
    if (sec != END) return io_fail(ACHR_ERR_PARSE, std::string(path) + ": missing ENDATA");
    if (lb.empty()) return io_fail(ACHR_ERR_PARSE, std::string(path) + ": no columns");
    const size_t nnz = vals.size(), n = lb.size();
    out->row_buf = (int32_t *)std::malloc(sizeof(int32_t) * (nnz ? nnz : 1));
    out->col_buf = (int32_t *)std::malloc(sizeof(int32_t) * (nnz ? nnz : 1));
    out->val_buf = (double *)std::malloc(sizeof(double) * (nnz ? nnz : 1));
    out->lb_buf = (double *)std::malloc(sizeof(double) * n);
    out->ub_buf = (double *)std::malloc(sizeof(double) * n);
    if (!out->row_buf || !out->col_buf || !out->val_buf || !out->lb_buf || !out->ub_buf) {
        achr_free_model(out);
        return io_fail(ACHR_ERR_NOMEM, "out of host memory reading MPS");
    }
    if (nnz) {
        std::memcpy(out->row_buf, rows.data(), sizeof(int32_t) * nnz);
        std::memcpy(out->col_buf, cols.data(), sizeof(int32_t) * nnz);
        std::memcpy(out->val_buf, vals.data(), sizeof(double) * nnz);
    }
    std::memcpy(out->lb_buf, lb.data(), sizeof(double) * n);
    std::memcpy(out->ub_buf, ub.data(), sizeof(double) * n);
    out->model.n_rxns = (int32_t)n;
    out->model.n_mets = nrows;
    out->model.nnz = (int64_t)nnz;
    out->model.row = out->row_buf;
    out->model.col = out->col_buf;
    out->model.val = out->val_buf;
    out->model.lb = out->lb_buf;
    out->model.ub = out->ub_buf;
    return ACHR_OK;
}

achr_status achr_read_warmup_csv(const char *path, int32_t n_rxns, double **warmup_out, int32_t *n_warmup_out) {
    if (!path || !warmup_out || !n_warmup_out || n_rxns <= 0) return io_fail(ACHR_ERR_INVALID, "bad argument");
    *warmup_out = nullptr;
    *n_warmup_out = 0;
    std::string data;
    if (!read_file(path, data)) return io_fail(ACHR_ERR_IO, std::string("cannot read warmup file ") + path);
    // Tokens are the non-empty runs between commas, as strtok(",") yields them
    // (ACHRCuda.cu:394-397, 406-410); a last token of only white space (the
    // line end) is not a value.
    std::vector<double> vals;
    int64_t W = -1;
    size_t pos = 0;
    int32_t row = 0;
    while (pos < data.size()) {
        size_t eol = data.find('\n', pos);
        if (eol == std::string::npos) eol = data.size();
        const char *b = data.data() + pos, *e = data.data() + eol;
        pos = eol + 1;
        // skip lines that are entirely white space
        const char *q = b;
        while (q < e && (*q == ' ' || *q == '\t' || *q == '\r')) ++q;
        if (q == e) continue;
        if (row >= n_rxns)
            return io_fail(ACHR_ERR_PARSE, std::string(path) + ": more than n_rxns=" + std::to_string(n_rxns) + " lines");
        int64_t count = 0;
        const char *t = b;
        while (t < e) {
            while (t < e && *t == ',') ++t;
            if (t >= e) break;
            const char *te = t;
            while (te < e && *te != ',') ++te;
            const char *ws = t;
            while (ws < te && (*ws == ' ' || *ws == '\t' || *ws == '\r')) ++ws;
            if (ws == te) {
                if (te == e) break;  // trailing white space only
                return io_fail(ACHR_ERR_PARSE, std::string(path) + ": empty value on line " + std::to_string(row + 1));
            }
            std::string tokstr(t, te);
            char *endp = nullptr;
            double v = std::strtod(tokstr.c_str(), &endp);
            while (endp && (*endp == ' ' || *endp == '\t' || *endp == '\r')) ++endp;
            if (!endp || *endp != '\0' || endp == tokstr.c_str())
                return io_fail(ACHR_ERR_PARSE, std::string(path) + ": bad value '" + tokstr + "' on line " +
                                                    std::to_string(row + 1));
            if (!std::isfinite(v))
                return io_fail(ACHR_ERR_PARSE, std::string(path) + ": non-finite value on line " + std::to_string(row + 1));
            vals.push_back(v);
            ++count;
            t = te;
        }
        if (W < 0) {
            W = count;
            if (W <= 0) return io_fail(ACHR_ERR_PARSE, std::string(path) + ": first line has no values");
            vals.reserve((size_t)W * (size_t)n_rxns);
        } else if (count != W) {
            return io_fail(ACHR_ERR_PARSE, std::string(path) + ": line " + std::to_string(row + 1) + " has " +
                                                std::to_string(count) + " values, expected " + std::to_string(W));
        }
        ++row;
    }
    if (row != n_rxns)
        return io_fail(ACHR_ERR_PARSE, std::string(path) + ": " + std::to_string(row) + " lines, expected n_rxns=" +
                                            std::to_string(n_rxns));
    if (W > std::numeric_limits<int32_t>::max()) return io_fail(ACHR_ERR_UNSUPPORTED, "too many warmup points");
    double *wm = (double *)std::malloc(sizeof(double) * (size_t)W * (size_t)n_rxns);
    if (!wm) return io_fail(ACHR_ERR_NOMEM, "out of host memory reading warmup");
    // line k holds reaction k across all points: column-major n x W (ACHRCuda.cu:409)
    for (int32_t k = 0; k < n_rxns; ++k)
        for (int64_t j = 0; j < W; ++j) wm[(size_t)j * (size_t)n_rxns + (size_t)k] = vals[(size_t)k * (size_t)W + (size_t)j];
    *warmup_out = wm;
    *n_warmup_out = (int32_t)W;
    return ACHR_OK;
}

// Exact "%f": round |v| * 10^6 to the nearest integer, ties to even, using the
// binary significand and exponent (|v| = m 2^e); values at or above 2^53,
// infinities and NaN go through snprintf.
int32_t achr_format_f(double v, char *buf) {
    if (!std::isfinite(v) || std::fabs(v) >= 9007199254740992.0) return (int32_t)std::snprintf(buf, 320, "%f", v);
    uint64_t bits;
    std::memcpy(&bits, &v, sizeof bits);
    const bool neg = (bits >> 63) != 0;
    const int bexp = (int)((bits >> 52) & 0x7FF);
    uint64_t mant = bits & 0xFFFFFFFFFFFFFull;
    int e;
    if (bexp == 0) e = -1074;
    else {
        mant |= 1ull << 52;
        e = bexp - 1075;
    }
    unsigned __int128 q;
    if (mant == 0) q = 0;
    else {
        const unsigned __int128 M = (unsigned __int128)mant * 1000000u;
        if (e >= 0) q = M << e;  // e == 0 only: |v| < 2^53 keeps e <= 0
        else {
            const int sh = -e;
            if (sh >= 100) q = 0;  // M < 2^73: value < 0.5 and never exactly 0.5
            else {
                q = M >> sh;
                const unsigned __int128 rem = M - (q << sh);
                const unsigned __int128 half = (unsigned __int128)1 << (sh - 1);
                if (rem > half || (rem == half && (q & 1))) ++q;
            }
        }
    }
    uint64_t ip = (uint64_t)(q / 1000000u);
    uint32_t fp = (uint32_t)(q % 1000000u);
    char tmp[32];
    int len = 0;
    do {
        tmp[len++] = (char)('0' + ip % 10);
        ip /= 10;
    } while (ip);
    int o = 0;
    if (neg) buf[o++] = '-';
    while (len) buf[o++] = tmp[--len];
    buf[o++] = '.';
    for (int k = 5; k >= 0; --k) {
        buf[o + k] = (char)('0' + fp % 10);
        fp /= 10;
    }
    o += 6;
    buf[o] = '\0';
    return o;
}

achr_status achr_write_points_csv(const char *path, const double *points, int32_t n_rxns, int32_t n_points,
                                  int32_t threads) {
    if (!path || (!points && (int64_t)n_rxns * n_points > 0) || n_rxns < 0 || n_points < 0)
        return io_fail(ACHR_ERR_INVALID, "bad argument");
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(ACHR_ERR_IO, std::string("cannot open ") + path + " for writing");
    if (threads <= 0) {
        unsigned hc = std::thread::hardware_concurrency();
        threads = hc ? (int32_t)hc : 1;
    }
    if (threads > 64) threads = 64;
    // Rows are formatted in blocks by `threads` workers, then written in order.
    const int32_t block_rows = n_points > 0 ? std::max<int32_t>(1, (int32_t)(4000000 / n_points)) : n_rxns;
    std::vector<std::string> bufs((size_t)threads);
    bool ok = true;
    for (int32_t r0 = 0; r0 < n_rxns && ok; r0 += block_rows * threads) {
        std::vector<std::thread> pool;
        for (int32_t t = 0; t < threads; ++t) {
            pool.emplace_back([&, t]() {
                std::string &s = bufs[(size_t)t];
                s.clear();
                const int32_t a = r0 + t * block_rows;
                const int32_t b = std::min<int32_t>(n_rxns, a + block_rows);
                char cell[320];
                for (int32_t i = a; i < b; ++i) {
                    const double *rowp = points + (size_t)i * (size_t)n_points;
                    for (int32_t j = 0; j < n_points; ++j) {
                        int32_t L = achr_format_f(rowp[j], cell);
                        s.append(cell, (size_t)L);
                        s.push_back(j + 1 < n_points ? ',' : '\n');
                    }
                    if (n_points == 0) s.push_back('\n');
                }
            });
        }
        for (auto &th : pool) th.join();
        for (int32_t t = 0; t < threads && ok; ++t)
            if (!bufs[(size_t)t].empty() && std::fwrite(bufs[(size_t)t].data(), 1, bufs[(size_t)t].size(), f) != bufs[(size_t)t].size())
                ok = false;
    }
    if (std::fclose(f) != 0) ok = false;
    if (!ok) return io_fail(ACHR_ERR_IO, std::string("write to ") + path + " failed");
    return ACHR_OK;
}

}  // extern "C"
