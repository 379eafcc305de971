/*
 * host_frontend.cpp — NRAPS input-file front end and mesh builder (host only).
 *
 * Keeps the reference's input format exactly, quirks included, so existing
 * input files parse identically:
 *   - scan_ascii_chunk (src/process_input.rs:44-83): '#' skips to the end of
 *     the line and the scanner then also steps over the first character of
 *     the next line; a key is the text from the line start to one character
 *     before the last '=' of the line (so "Key = v" needs the space); keys are
 *     trimmed and lower-cased; a repeated key appends its value after a space.
 *   - get_index (src/process_input.rs:13-42): a key is identified only by its
 *     last two characters and its length.
 *   - process_input (src/process_input.rs:85-175): rodpitch is stored as
 *     pitch - diameter; inv_sigtr = 1/(sigt - mu*sigs) in f32; `solution` is
 *     the bool "Solution != 1"; `solver` maps "1"/"2"/"3" else LinAlg.
 *   - mesh_gen (src/main.rs:85-143): MatID expanded by MPFR/MPWR, MPWR cells
 *     removed at each assembly junction (index recomputed from the shrinking
 *     length), MPWR/2 cells trimmed at each edge, f32 running cell bounds.
 * Where the reference panics (unparsable value, key shorter than two
 * characters, empty MatID) this returns NRAPS_ERR_PARSE / NRAPS_ERR_INVALID.
 */
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/nraps_gpu.h"
#include "host_common.hpp"

namespace {

int get_index(const std::string& key) {
    size_t n = key.size();
    std::string k2 = key.substr(n - 2, 2);
    struct E { const char* k; size_t len; int idx; };
    static const E table[] = {
        {"lk", 5, 0},  {"es", 8, 1},  {"ps", 12, 2}, {"ns", 11, 3}, {"es", 9, 4},
        {"ip", 4, 5},  {"ss", 6, 6},  {"ds", 7, 7},  {"ia", 6, 8},  {"ch", 8, 9},
        {"fr", 4, 10}, {"wr", 4, 11}, {"dl", 6, 12}, {"dr", 6, 13}, {"gt", 4, 14},
        {"gs", 4, 15}, {"mu", 2, 16}, {"ga", 4, 17}, {"gf", 4, 18}, {"ut", 3, 19},
        {"it", 4, 20}, {"at", 4, 21}, {"id", 5, 22}, {"on", 8, 23}, {"er", 6, 24},
    };
    for (const E& e : table)
        if (n == e.len && k2 == e.k) return e.idx;
    return 25;
}

std::string trim(const std::string& s) {
    /* Rust str::trim strips Unicode White_Space; for ASCII input that is
       space, \t, \n, \v, \f, \r */
    auto ws = [](unsigned char c) { return c == ' ' || (c >= '\t' && c <= '\r'); };
    size_t a = 0, b = s.size();
    while (a < b && ws(s[a])) ++a;
    while (b > a && ws(s[b - 1])) --b;
    return s.substr(a, b - a);
}

std::vector<std::string> split_ws(const std::string& s) {
    std::vector<std::string> out;
    size_t i = 0, n = s.size();
    auto ws = [](unsigned char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\f' || c == '\r'; };
    while (i < n) {
        while (i < n && ws(s[i])) ++i;
        size_t j = i;
        while (j < n && !ws(s[j])) ++j;
        if (j > i) out.push_back(s.substr(i, j - i));
        i = j;
    }
    return out;
}

/* scan_ascii_chunk */
int scan(const char* buf, size_t end, std::string temp[26]) {
    size_t pos = 0, line_start = 0, name_end = 0, val_start = 0;
    while (pos < end) {
        char c = buf[pos];
        if (c == '#') {
            /* skip_line: stop at '\n' or end, return one past it */
            while (pos < end && buf[pos] != '\n') ++pos;
            pos = pos + 1;
            line_start = pos;
        } else if (c == '=') {
            name_end = pos - 1;
            val_start = pos + 1;
        } else if (c == '\n') {
            if (name_end > line_start) {
                std::string key = trim(std::string(buf + line_start, name_end - line_start));
                for (char& ch : key) if (ch >= 'A' && ch <= 'Z') ch = (char)(ch - 'A' + 'a');
                std::string value = val_start <= pos ? trim(std::string(buf + val_start, pos - val_start)) : std::string();
                if (key.size() < 2) {
                    nraps_host::set_error("input key '" + key + "' is shorter than two characters");
                    return NRAPS_ERR_PARSE;
                }
                temp[get_index(key)] += " " + value;
            }
            line_start = pos + 1;
        }
        pos += 1;
    }
    return NRAPS_OK;
}

bool parse_uint(const std::string& s0, uint64_t maxv, uint64_t* out) {
    std::string s = trim(s0);
    size_t i = 0;
    if (i < s.size() && s[i] == '+') ++i;
    if (i >= s.size()) return false;
    uint64_t v = 0;
    for (; i < s.size(); ++i) {
        if (s[i] < '0' || s[i] > '9') return false;
        uint64_t d = (uint64_t)(s[i] - '0');
        if (v > (maxv - d) / 10) return false;
        v = v * 10 + d;
    }
    *out = v;
    return true;
}

bool parse_f32(const std::string& s0, float* out) {
    std::string s = trim(s0);
    if (s.empty()) return false;
    for (char c : s) if (c == 'x' || c == 'X' || c == ' ') return false; /* no hex floats */
    errno = 0;
    char* endp = nullptr;
    float v = std::strtof(s.c_str(), &endp);
    if (endp != s.c_str() + s.size()) return false;
    *out = v;
    return true;
}

int fail_parse(const char* what, const std::string& text) {
    nraps_host::set_error(std::string("cannot parse ") + what + " from '" + trim(text) + "'");
    return NRAPS_ERR_PARSE;
}

template <class T> T* dup_vec(const std::vector<T>& v) {
    T* p = (T*)std::malloc(std::max<size_t>(1, v.size()) * sizeof(T));
    if (p && !v.empty()) std::memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

int parse_list(const std::string& s, const char* what, std::vector<float>& out) {
    for (const std::string& tok : split_ws(s)) {
        float v;
        if (!parse_f32(tok, &v)) return fail_parse(what, tok);
        out.push_back(v);
    }
    return NRAPS_OK;
}

} // namespace

extern "C" {

int nraps_process_input_text(const char* text, uint64_t len, nraps_input** out) {
    if (!text || !out) { nraps_host::set_error("null argument"); return NRAPS_ERR_INVALID; }
    *out = nullptr;
    std::string temp[26];
    int st = scan(text, (size_t)len, temp);
    if (st) return st;
    nraps_input* in = (nraps_input*)std::calloc(1, sizeof(nraps_input));
    if (!in) return NRAPS_ERR_NOMEM;
    nraps_variables& v = in->variables;
    uint64_t u;
    float f, f2;
#define PU(idx, field, maxv, name) \
    if (!parse_uint(temp[idx], maxv, &u)) { nraps_input_free(in); return fail_parse(name, temp[idx]); } \
    v.field = (decltype(v.field))u;
    PU(0, analk, 255, "Analk")
    PU(1, mattypes, 255, "MatTypes")
    PU(2, energygroups, 255, "EnergyGroups")
    PU(3, generations, UINT64_MAX, "Generations")
    PU(4, histories, UINT64_MAX, "Histories")
    PU(5, skip, UINT64_MAX, "Skip")
    PU(6, numass, 255, "NumAss")
    PU(7, numrods, 255, "NumRods")
    if (!parse_f32(temp[8], &f)) { nraps_input_free(in); return fail_parse("RodDia", temp[8]); }
    v.roddia = f;
    if (!parse_f32(temp[9], &f2)) { nraps_input_free(in); return fail_parse("RodPitch", temp[9]); }
    v.rodpitch = f2 - f;                                      /* :102 */
    PU(10, mpfr, UINT64_MAX, "MPFR")
    PU(11, mpwr, UINT64_MAX, "MPWR")
#undef PU
    if (!parse_f32(temp[12], &v.boundl)) { nraps_input_free(in); return fail_parse("BoundL", temp[12]); }
    if (!parse_f32(temp[13], &v.boundr)) { nraps_input_free(in); return fail_parse("BoundR", temp[13]); }
    in->delta_x.fuel = v.roddia / (float)v.mpfr;              /* :109-112 */
    in->delta_x.water = v.rodpitch / (float)v.mpwr;

    std::vector<float> lists[8];
    const char* names[8] = {"SigT", "SigS", "mu", "SigA", "SigF", "nuT", "ChiT", "Scat"};
    for (int i = 0; i < 8; ++i) {
        st = parse_list(temp[14 + i], names[i], lists[i]);
        if (st) { nraps_input_free(in); return st; }
    }
    std::vector<float> inv(lists[0].size());
    for (size_t i = 0; i < lists[0].size(); ++i) {
        float mu = i < lists[2].size() ? lists[2][i] : 0.0f;  /* Rust would panic */
        float ss = i < lists[1].size() ? lists[1][i] : 0.0f;
        inv[i] = 1.0f / (lists[0][i] - mu * ss);               /* :152-156 */
    }
    in->sigt = dup_vec(lists[0]); in->n_sigt = lists[0].size();
    in->sigs = dup_vec(lists[1]); in->n_sigs = lists[1].size();
    in->mu = dup_vec(lists[2]);   in->n_mu = lists[2].size();
    in->siga = dup_vec(lists[3]); in->n_siga = lists[3].size();
    in->sigf = dup_vec(lists[4]); in->n_sigf = lists[4].size();
    in->nut = dup_vec(lists[5]);  in->n_nut = lists[5].size();
    in->chit = dup_vec(lists[6]); in->n_chit = lists[6].size();
    in->scat_matrix = dup_vec(lists[7]); in->n_scat = lists[7].size();
    in->inv_sigtr = dup_vec(inv); in->n_inv_sigtr = inv.size();

    std::vector<uint8_t> mat;
    for (const std::string& tok : split_ws(temp[22])) {
        if (!parse_uint(tok, 255, &u)) { nraps_input_free(in); return fail_parse("MatID", tok); }
        mat.push_back((uint8_t)u);
    }
    in->matid = dup_vec(mat); in->n_matid = mat.size();
    if (!parse_uint(temp[23], 255, &u)) { nraps_input_free(in); return fail_parse("Solution", temp[23]); }
    in->solution = (u != 1) ? 1 : 0;
    std::string sv = trim(temp[24]);
    in->solver = sv == "1" ? 1 : sv == "2" ? 2 : sv == "3" ? 3 : 0;
    *out = in;
    return NRAPS_OK;
}

int nraps_process_input(const char* path, nraps_input** out) {
    if (!path || !out) { nraps_host::set_error("null argument"); return NRAPS_ERR_INVALID; }
    FILE* fp = std::fopen(path, "rb");
    if (!fp) { nraps_host::set_error(std::string("Unable to read the file ") + path); return NRAPS_ERR_IO; }
    std::string data;
    char buf[1 << 16];
    size_t n;
    while ((n = std::fread(buf, 1, sizeof buf, fp)) > 0) data.append(buf, n);
    std::fclose(fp);
    return nraps_process_input_text(data.data(), data.size(), out);
}

void nraps_input_free(nraps_input* in) {
    if (!in) return;
    float* arrs[] = {in->sigt, in->sigs, in->mu, in->siga, in->sigf, in->nut, in->chit,
                     in->scat_matrix, in->inv_sigtr};
    for (float* a : arrs) std::free(a);
    std::free(in->matid);
    std::free(in);
}

int nraps_mesh_gen(const uint8_t* matid, uint64_t n_matid, const nraps_variables* v,
                   const nraps_delta_x* dx, nraps_meshbuf** out) {
    if (!matid || !v || !dx || !out) { nraps_host::set_error("null argument"); return NRAPS_ERR_INVALID; }
    *out = nullptr;
    std::vector<uint8_t> temp;
    for (uint64_t i = 0; i < n_matid; ++i) {
        uint64_t reps = (matid[i] == 0 || matid[i] == 1) ? v->mpfr : v->mpwr;
        temp.insert(temp.end(), reps, matid[i]);
    }
    /* remove the extra water meshes at each assembly junction (main.rs:99-103) */
    for (uint64_t a = 1; a < v->numass; ++a)
        for (uint64_t k = 0; k < v->mpwr; ++k) {
            uint64_t idx = (a * (uint64_t)temp.size()) / v->numass;
            if (idx >= temp.size()) { nraps_host::set_error("mesh_gen: junction index out of range"); return NRAPS_ERR_INVALID; }
            temp.erase(temp.begin() + (ptrdiff_t)idx);
        }
    uint64_t half = v->mpwr / 2;                                       /* :107-108 */
    if (temp.size() < 2 * half) { nraps_host::set_error("mesh_gen: fewer cells than the edge trim"); return NRAPS_ERR_INVALID; }
    temp.erase(temp.begin(), temp.begin() + (ptrdiff_t)half);
    temp.resize(temp.size() - half);
    if (temp.empty()) { nraps_host::set_error("mesh_gen: empty mesh"); return NRAPS_ERR_INVALID; }

    nraps_meshbuf* m = (nraps_meshbuf*)std::calloc(1, sizeof(nraps_meshbuf));
    if (!m) return NRAPS_ERR_NOMEM;
    size_t n = temp.size();
    m->n_cells = n;
    m->matid = (uint8_t*)std::malloc(n);
    m->delta_x = (float*)std::malloc(n * 4);
    m->mesh_left = (float*)std::malloc(n * 4);
    m->mesh_right = (float*)std::malloc(n * 4);
    std::vector<uint64_t> fuel;
    float left = 0.0f;
    for (size_t i = 0; i < n; ++i) {
        bool is_fuel = temp[i] == 0 || temp[i] == 1;
        float d = is_fuel ? dx->fuel : dx->water;
        m->matid[i] = temp[i];
        m->delta_x[i] = d;
        m->mesh_left[i] = left;
        m->mesh_right[i] = left + d;
        left += d;
        if (is_fuel) fuel.push_back(i);
    }
    m->fuel_indices = dup_vec(fuel);
    m->n_fuel = fuel.size();
    *out = m;
    return NRAPS_OK;
}

void nraps_meshbuf_free(nraps_meshbuf* m) {
    if (!m) return;
    std::free(m->matid); std::free(m->delta_x); std::free(m->mesh_left);
    std::free(m->mesh_right); std::free(m->fuel_indices);
    std::free(m);
}

int nraps_problem_view(const nraps_input* in, const nraps_meshbuf* mesh, nraps_problem* out) {
    if (!in || !mesh || !out) { nraps_host::set_error("null argument"); return NRAPS_ERR_INVALID; }
    std::memset(out, 0, sizeof *out);
    out->variables = in->variables;
    out->delta_x = in->delta_x;
    nraps_xsdata& x = out->xsdata;
    x.sigt = in->sigt; x.sigs = in->sigs; x.mu = in->mu; x.siga = in->siga;
    x.sigf = in->sigf; x.nut = in->nut; x.chit = in->chit;
    x.scat_matrix = in->scat_matrix; x.inv_sigtr = in->inv_sigtr;
    x.n_xs = in->n_sigt; x.n_scat = in->n_scat;
    out->mesh.matid = mesh->matid; out->mesh.delta_x = mesh->delta_x;
    out->mesh.mesh_left = mesh->mesh_left; out->mesh.mesh_right = mesh->mesh_right;
    out->mesh.n_cells = mesh->n_cells;
    out->fuel_indices = mesh->fuel_indices;
    out->n_fuel = mesh->n_fuel;
    out->k_new = 1.0f;                                   /* main.rs:337 */
    return NRAPS_OK;
}

const char* nraps_status_string(int s) {
    switch (s) {
        case NRAPS_OK: return "ok";
        case NRAPS_ERR_INVALID: return "invalid argument";
        case NRAPS_ERR_CUDA: return "CUDA error";
        case NRAPS_ERR_NOMEM: return "out of memory";
        case NRAPS_ERR_NO_DEVICE: return "no CUDA device";
        case NRAPS_ERR_IO: return "I/O error";
        case NRAPS_ERR_PARSE: return "parse error";
        case NRAPS_ERR_CAPACITY: return "bank or queue capacity exceeded";
        case NRAPS_ERR_EMPTY_BANK: return "fission bank empty";
        case NRAPS_ERR_NOT_FOUND: return "not found";
        case NRAPS_ERR_PENDING: return "pending";
        case NRAPS_ERR_CAPPED: return "history event cap reached";
        case NRAPS_ERR_REJECTED: return "rejected: exceeds memory budget";
        case NRAPS_ERR_UNSUPPORTED: return "unsupported: solver not in this library";
        default: return "unknown status";
    }
}

} /* extern "C" */
