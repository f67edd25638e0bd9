// Settings of a simulation: a YAML-subset reader and the reference's schema with its
// defaults (Settings::read, src/settings.cpp:314-594; defaults of src/default-settings.yml).
//
// The reader handles what FeeLLGood settings files use: block maps and sequences by
// indentation, flow sequences [a, b], flow maps {k: v} (so JSON settings work, as
// ci-tests/full_test.py feeds them), plain and quoted scalars, and # comments.
// Expressions of x, y, z or t (the reference evaluates them with Duktape) are not
// supported: initial magnetisation and applied field must be numbers or a .sol file.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "fg_host.h"
#include "host_settings.h"

namespace fgh {

// ---------------------------------------------------------------------------------
// YAML subset

std::shared_ptr<YNode> YNode::get(const std::string &k) const {
    for (auto &p : map)
        if (p.first == k) return p.second;
    return nullptr;
}

namespace {

struct Line {
    int indent;
    std::string text;  // without indent, comment stripped, right-trimmed
    int lineno;
};

std::string strip_comment(const std::string &s) {
    bool sq = false, dq = false;
    for (size_t i = 0; i < s.size(); i++) {
        const char c = s[i];
        if (c == '\'' && !dq) sq = !sq;
        else if (c == '"' && !sq) dq = !dq;
        else if (c == '#' && !sq && !dq && (i == 0 || std::isspace((unsigned char)s[i - 1]))) return s.substr(0, i);
    }
    return s;
}
std::string rtrim(const std::string &s) {
    size_t e = s.find_last_not_of(" \t\r\n");
    return e == std::string::npos ? "" : s.substr(0, e + 1);
}
std::string trim(const std::string &s) {
    size_t b = s.find_first_not_of(" \t\r\n");
    return b == std::string::npos ? "" : rtrim(s.substr(b));
}

struct FlowParser {
    const std::string &s;
    size_t p = 0;
    explicit FlowParser(const std::string &str) : s(str) {}
    void ws() {
        while (p < s.size() && std::isspace((unsigned char)s[p])) p++;
    }
    std::shared_ptr<YNode> value() {
        ws();
        if (p >= s.size()) throw YamlError("unexpected end of flow value");
        if (s[p] == '[') {
            auto n = std::make_shared<YNode>();
            n->kind = YNode::SEQ;
            p++;
            ws();
            if (p < s.size() && s[p] == ']') { p++; return n; }
            for (;;) {
                n->seq.push_back(value());
                ws();
                if (p < s.size() && s[p] == ',') { p++; continue; }
                if (p < s.size() && s[p] == ']') { p++; break; }
                throw YamlError("expected , or ] in flow sequence");
            }
            return n;
        }
        if (s[p] == '{') {
            auto n = std::make_shared<YNode>();
            n->kind = YNode::MAP;
            p++;
            ws();
            if (p < s.size() && s[p] == '}') { p++; return n; }
            for (;;) {
                ws();
                std::string k = scalar_text(true);
                ws();
                if (p >= s.size() || s[p] != ':') throw YamlError("expected : in flow map");
                p++;
                n->map.push_back({k, value()});
                ws();
                if (p < s.size() && s[p] == ',') { p++; continue; }
                if (p < s.size() && s[p] == '}') { p++; break; }
                throw YamlError("expected , or } in flow map");
            }
            return n;
        }
        auto n = std::make_shared<YNode>();
        n->kind = YNode::SCALAR;
        const bool quoted = s[p] == '"' || s[p] == '\'';
        n->scalar = scalar_text(false);
        n->quoted = quoted;
        if (!quoted && (n->scalar == "null" || n->scalar == "~" || n->scalar.empty())) n->kind = YNode::NUL;
        return n;
    }
    std::string scalar_text(bool key) {
        ws();
        if (p < s.size() && (s[p] == '"' || s[p] == '\'')) {
            const char q = s[p++];
            std::string out;
            while (p < s.size() && s[p] != q) {
                if (s[p] == '\\' && q == '"' && p + 1 < s.size()) {
                    p++;
                    out += s[p] == 'n' ? '\n' : s[p];
                } else out += s[p];
                p++;
            }
            if (p >= s.size()) throw YamlError("unterminated quoted scalar");
            p++;
            return out;
        }
        size_t b = p;
        while (p < s.size() && s[p] != ',' && s[p] != ']' && s[p] != '}' && !(key && s[p] == ':')) p++;
        return trim(s.substr(b, p - b));
    }
};

std::shared_ptr<YNode> parse_inline(const std::string &v) {
    FlowParser fp(v);
    auto n = fp.value();
    fp.ws();
    if (fp.p != v.size()) throw YamlError("trailing characters after value: " + v);
    return n;
}

// position of the key separator ": " (or ':' at end), outside quotes and brackets
size_t key_colon(const std::string &t) {
    bool sq = false, dq = false;
    int depth = 0;
    for (size_t i = 0; i < t.size(); i++) {
        const char c = t[i];
        if (c == '\'' && !dq) sq = !sq;
        else if (c == '"' && !sq) dq = !dq;
        else if (!sq && !dq) {
            if (c == '[' || c == '{') depth++;
            else if (c == ']' || c == '}') depth--;
            else if (c == ':' && depth == 0 && (i + 1 == t.size() || t[i + 1] == ' ' || t[i + 1] == '\t')) return i;
        }
    }
    return std::string::npos;
}

struct BlockParser {
    std::vector<Line> L;
    size_t i = 0;
    std::shared_ptr<YNode> block(int indent) {
        if (i >= L.size() || L[i].indent < indent) {
            auto n = std::make_shared<YNode>();
            n->kind = YNode::NUL;
            return n;
        }
        const int ind = L[i].indent;
        if (L[i].text.rfind("- ", 0) == 0 || L[i].text == "-") {
            auto n = std::make_shared<YNode>();
            n->kind = YNode::SEQ;
            while (i < L.size() && L[i].indent == ind && (L[i].text.rfind("- ", 0) == 0 || L[i].text == "-")) {
                std::string rest = L[i].text == "-" ? "" : trim(L[i].text.substr(2));
                const int lineno = L[i].lineno;
                i++;
                if (rest.empty()) n->seq.push_back(block(ind + 1));
                else if (key_colon(rest) != std::string::npos && rest[0] != '[' && rest[0] != '{') {
                    // a map starting on the dash line
                    Line first{ind + 2, rest, lineno};
                    L.insert(L.begin() + i, first);
                    n->seq.push_back(block(ind + 2));
                } else n->seq.push_back(parse_inline(rest));
            }
            return n;
        }
        auto n = std::make_shared<YNode>();
        n->kind = YNode::MAP;
        while (i < L.size() && L[i].indent == ind) {
            const std::string &t = L[i].text;
            const size_t c = key_colon(t);
            if (c == std::string::npos) {
                if (L.size() == 1 || t[0] == '{' || t[0] == '[') {
                    auto v = parse_inline(t);
                    i++;
                    return v;
                }
                throw YamlError("line " + std::to_string(L[i].lineno) + ": expected 'key: value'");
            }
            std::string key = trim(t.substr(0, c));
            if (key.size() >= 2 && (key[0] == '"' || key[0] == '\'')) key = key.substr(1, key.size() - 2);
            const std::string val = trim(t.substr(c + 1));
            i++;
            if (val.empty()) {
                if (i < L.size() && L[i].indent > ind) n->map.push_back({key, block(L[i].indent)});
                else if (i < L.size() && L[i].indent == ind && L[i].text.rfind("- ", 0) == 0)
                    n->map.push_back({key, block(ind)});  // sequence at the key's indentation
                else {
                    auto z = std::make_shared<YNode>();
                    z->kind = YNode::NUL;
                    n->map.push_back({key, z});
                }
            } else n->map.push_back({key, parse_inline(val)});
        }
        return n;
    }
};

}  // namespace

std::shared_ptr<YNode> yaml_parse(const std::string &text) {
    // whole document in flow style (JSON)
    const std::string t = trim(text);
    if (!t.empty() && t[0] == '{') {
        std::string one;
        std::istringstream in(text);
        std::string line;
        while (std::getline(in, line)) one += strip_comment(line) + " ";
        return parse_inline(trim(one));
    }
    BlockParser bp;
    std::istringstream in(text);
    std::string line;
    int lineno = 0;
    std::string pending;
    int pending_indent = 0, pending_line = 0, depth = 0;
    while (std::getline(in, line)) {
        lineno++;
        std::string s = rtrim(strip_comment(line));
        if (trim(s).empty()) continue;
        if (trim(s) == "---") continue;
        int ind = 0;
        while (ind < (int)s.size() && s[ind] == ' ') ind++;
        std::string body = s.substr(ind);
        if (!pending.empty()) {
            pending += " " + body;
        } else {
            pending = body;
            pending_indent = ind;
            pending_line = lineno;
        }
        for (char ch : body) {
            if (ch == '[' || ch == '{') depth++;
            else if (ch == ']' || ch == '}') depth--;
        }
        if (depth <= 0) {
            bp.L.push_back({pending_indent, pending, pending_line});
            pending.clear();
            depth = 0;
        }
    }
    if (!pending.empty()) throw YamlError("unterminated flow collection");
    if (bp.L.empty()) {
        auto n = std::make_shared<YNode>();
        n->kind = YNode::NUL;
        return n;
    }
    auto n = bp.block(bp.L[0].indent);
    if (bp.i != bp.L.size()) throw YamlError("line " + std::to_string(bp.L[bp.i].lineno) + ": bad indentation");
    return n;
}

// ---------------------------------------------------------------------------------
// Settings

namespace {

bool is_null(const std::shared_ptr<YNode> &n) { return !n || n->kind == YNode::NUL; }

double to_num(const std::shared_ptr<YNode> &n, const std::string &what) {
    if (!n || n->kind != YNode::SCALAR) throw SettingsError(what + " should be a number");
    char *end = nullptr;
    const double v = std::strtod(n->scalar.c_str(), &end);
    if (end == n->scalar.c_str() || *end != '\0')
        throw SettingsError(what + " = '" + n->scalar + "' is not a number (expressions are not supported)");
    return v;
}
bool to_bool(const std::shared_ptr<YNode> &n, const std::string &what) {
    if (!n || n->kind != YNode::SCALAR) throw SettingsError(what + " should be true or false");
    if (n->scalar == "true" || n->scalar == "True" || n->scalar == "1") return true;
    if (n->scalar == "false" || n->scalar == "False" || n->scalar == "0") return false;
    throw SettingsError(what + " should be true or false");
}
void to_vec(const std::shared_ptr<YNode> &n, double *v, bool normalize, const std::string &what) {
    if (!n || n->kind != YNode::SEQ) throw SettingsError("vectors should be YAML sequences (" + what + ")");
    if (n->seq.size() != 3) throw SettingsError("vectors should have three components (" + what + ")");
    for (int k = 0; k < 3; k++) v[k] = to_num(n->seq[k], what);
    if (normalize) {
        const double s = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (s > 0)
            for (int k = 0; k < 3; k++) v[k] /= s;
    }
}

void apply_yaml(Settings &S, const std::shared_ptr<YNode> &y) {
    if (is_null(y)) return;
    if (y->kind != YNode::MAP) throw SettingsError("settings should be a map");
    if (auto o = y->get("outputs"); !is_null(o)) {
        if (o->kind != YNode::MAP) throw SettingsError("outputs should be a map.");
        if (auto d = o->get("directory"); d && d->kind == YNode::SCALAR) {
            S.out_dir = d->scalar.empty() ? "." : d->scalar;
            if (S.out_dir.size() > 1 && S.out_dir.back() == '/') S.out_dir.pop_back();
        }
        if (auto d = o->get("file_basename"); d && d->kind == YNode::SCALAR) S.sim_name = d->scalar;
        if (auto d = o->get("evol_time_step"); !is_null(d)) S.evol_time_step = to_num(d, "outputs.evol_time_step");
        if (auto d = o->get("final_time"); !is_null(d)) S.final_time = to_num(d, "outputs.final_time");
        if (auto d = o->get("mag_config_every"); !is_null(d)) {
            if (d->scalar == "true") throw SettingsError("outputs.mag_config_every should be an integer or `false'.");
            if (d->scalar == "false") S.save_period = 0;
            else S.save_period = std::max(0, (int)to_num(d, "outputs.mag_config_every"));
        }
        if (auto d = o->get("evol_columns"); !is_null(d)) {
            if (d->kind != YNode::SEQ) throw SettingsError("outputs.evol_columns should be a sequence.");
            S.evol_columns.clear();
            for (auto &c : d->seq) S.evol_columns.push_back(c->scalar);
        }
        if (auto d = o->get("metadata"); !is_null(d)) {
            if (d->kind != YNode::MAP) throw SettingsError("outputs.metadata should be a map.");
            for (auto &kv : d->map) {
                bool found = false;
                for (auto &it : S.metadata)
                    if (it.first == kv.first) { it.second = kv.second->scalar; found = true; }
                if (!found) S.metadata.push_back({kv.first, kv.second->scalar});
            }
        }
    }
    if (auto m = y->get("mesh"); !is_null(m)) {
        if (m->kind != YNode::MAP) throw SettingsError("mesh should be a map.");
        if (auto d = m->get("filename"); d && d->kind == YNode::SCALAR) S.mesh_file = d->scalar;
        if (auto d = m->get("length_unit"); !is_null(d)) {
            S.length_unit = to_num(d, "mesh.length_unit");
            if (S.length_unit <= 0) throw SettingsError("mesh.length_unit should be positive.");
        }
        if (auto v = m->get("volume_regions"); !is_null(v)) {
            if (v->kind != YNode::MAP) throw SettingsError("mesh.volume_regions should be a map.");
            for (auto &kv : v->map) {
                VolRegion r = S.vol_default;
                r.name = kv.first;
                auto R = kv.second;
                if (!is_null(R)) {
                    bool has_ms = false, has_js = false;
                    if (auto d = R->get("Ae"); !is_null(d)) r.Ae = to_num(d, kv.first + ".Ae");
                    if (auto d = R->get("Ms"); !is_null(d)) { r.Ms = to_num(d, kv.first + ".Ms"); has_ms = true; }
                    if (auto d = R->get("Js"); !is_null(d)) { r.Ms = to_num(d, kv.first + ".Js") / 1.25663706127e-6; has_js = true; }
                    if (has_ms && has_js) throw SettingsError("Ms and Js should not be both defined in the same region.");
                    if (auto d = R->get("K"); !is_null(d)) r.K = to_num(d, kv.first + ".K");
                    if (auto d = R->get("uk"); !is_null(d)) to_vec(d, r.uk, true, kv.first + ".uk");
                    if (auto d = R->get("K3"); !is_null(d)) r.K3 = to_num(d, kv.first + ".K3");
                    if (auto d = R->get("ex"); !is_null(d)) to_vec(d, r.ex, true, kv.first + ".ex");
                    if (auto d = R->get("ey"); !is_null(d)) to_vec(d, r.ey, true, kv.first + ".ey");
                    if (auto d = R->get("ez"); !is_null(d)) to_vec(d, r.ez, true, kv.first + ".ez");
                    if (auto d = R->get("alpha_LLG"); !is_null(d)) r.alpha = to_num(d, kv.first + ".alpha_LLG");
                    if (auto d = R->get("sigma"); !is_null(d)) r.sigma = to_num(d, kv.first + ".sigma");
                    if (auto d = R->get("dens_state"); !is_null(d)) r.dens_state = to_num(d, kv.first + ".dens_state");
                    if (auto d = R->get("P"); !is_null(d)) r.P = to_num(d, kv.first + ".P");
                    if (auto d = R->get("l_sd"); !is_null(d)) r.lsd = to_num(d, kv.first + ".l_sd");
                    if (auto d = R->get("l_sf"); !is_null(d)) r.lsf = to_num(d, kv.first + ".l_sf");
                }
                if (kv.first == "__default__") S.vol_default = r;
                else S.vol.push_back(r);
            }
        }
        if (auto v = m->get("surface_regions"); !is_null(v)) {
            if (v->kind != YNode::MAP) throw SettingsError("mesh.surface_regions should be a map.");
            for (auto &kv : v->map) {
                SurfRegion r = S.surf_default;
                r.name = kv.first;
                auto R = kv.second;
                if (!is_null(R)) {
                    if (auto d = R->get("suppress_charges"); !is_null(d)) r.suppress_charges = to_bool(d, kv.first + ".suppress_charges");
                    if (auto d = R->get("Ks"); !is_null(d)) r.Ks = to_num(d, kv.first + ".Ks");
                    if (auto d = R->get("uk"); !is_null(d)) to_vec(d, r.uk, true, kv.first + ".uk");
                    if (auto d = R->get("jn"); !is_null(d)) r.jn = to_num(d, kv.first + ".jn");
                    if (auto d = R->get("V"); !is_null(d)) r.V = to_num(d, kv.first + ".V");
                    if (auto d = R->get("uP"); !is_null(d)) to_vec(d, r.uP, true, kv.first + ".uP");
                    if (auto d = R->get("s"); !is_null(d)) to_vec(d, r.s, false, kv.first + ".s");
                }
                if (kv.first == "__default__") S.surf_default = r;
                else S.surf.push_back(r);
            }
        }
    }
    if (auto d = y->get("initial_magnetization"); !is_null(d)) {
        if (d->kind == YNode::SCALAR) {
            S.restore_file = d->scalar;
            S.init_from_file = true;
        } else if (d->kind == YNode::SEQ) {
            to_vec(d, S.m0, true, "initial_magnetization");
            S.init_from_file = false;
        } else throw SettingsError("initial_magnetization should be a file name or a vector of expressions.");
    }
    if (auto d = y->get("initial_time"); !is_null(d)) S.initial_time = to_num(d, "initial_time");
    if (auto d = y->get("recentering"); !is_null(d)) {
        if (auto e = d->get("enable"); !is_null(e)) S.recenter = to_bool(e, "recentering.enable");
        if (auto e = d->get("direction"); !is_null(e)) {
            const std::string v = e->scalar;
            if (v == "X" || v == "x") S.recenter_dir = 0;
            else if (v == "Y" || v == "y") S.recenter_dir = 1;
            else if (v == "Z" || v == "z") S.recenter_dir = 2;
            else throw SettingsError("recentering.direction should be X, Y or Z");
        }
        if (auto e = d->get("threshold"); !is_null(e)) S.recenter_threshold = to_num(e, "recentering.threshold");
    }
    if (auto d = y->get("Bext"); !is_null(d)) {
        if (d->kind != YNode::SEQ) throw SettingsError("Bext should be a vector of numbers (expressions of t are not supported)");
        to_vec(d, S.Bext, false, "Bext");
    }
    if (auto d = y->get("spin_accumulation"); !is_null(d)) {
        if (auto e = d->get("enable"); !is_null(e)) S.spin_acc = to_bool(e, "spin_accumulation.enable");
        if (auto e = d->get("V_file"); !is_null(e)) S.V_file = to_bool(e, "spin_accumulation.V_file");
    }
    if (auto s = y->get("finite_element_solver"); !is_null(s)) {
        if (auto d = s->get("max(iter)"); !is_null(d)) S.max_iter = (int)to_num(d, "max(iter)");
        if (auto d = s->get("tolerance"); !is_null(d)) S.tol = to_num(d, "tolerance");
    }
    if (auto s = y->get("time_integration"); !is_null(s)) {
        if (auto d = s->get("max(du)"); !is_null(d)) S.dumax = to_num(d, "max(du)");
        if (auto d = s->get("min(dt)"); !is_null(d)) S.dt_min = to_num(d, "min(dt)");
        if (auto d = s->get("max(dt)"); !is_null(d)) S.dt_max = to_num(d, "max(dt)");
    }
    if (auto g = y->get("gpu"); !is_null(g)) {  // options of this build (ignored by the reference)
        if (auto d = g->get("precision"); !is_null(d)) S.gpu_precision = d->scalar == "fp32_refine" ? 1 : 0;
        if (auto d = g->get("learned_guess"); !is_null(d)) S.gpu_learned = to_bool(d, "gpu.learned_guess");
        if (auto d = g->get("demag"); !is_null(d)) S.gpu_demag = d->scalar == "direct" ? 1 : (d->scalar == "fmm" ? 2 : 0);
        if (auto d = g->get("one_gauss_point"); !is_null(d)) S.one_gauss_point = to_bool(d, "gpu.one_gauss_point");
        if (auto d = g->get("checkpoint_every"); !is_null(d)) {
            const double n = to_num(d, "gpu.checkpoint_every");
            if (!(n >= 0) || n != std::floor(n)) throw SettingsError("gpu.checkpoint_every must be a count >= 0");
            S.checkpoint_every = (int)n;
        }
        if (auto d = g->get("resume"); !is_null(d)) S.resume_file = d->scalar;
        auto count = [&](const char *key, int &out) {
            if (auto d = g->get(key); !is_null(d)) {
                const double n = to_num(d, std::string("gpu.") + key);
                if (!(n >= 0) || n != std::floor(n)) throw SettingsError(std::string("gpu.") + key + " must be a count >= 0");
                out = (int)n;
            }
        };
        count("solver_lanes_per_row", S.solver_lpr);
        count("solver_blocks", S.solver_blocks);
        count("solver_threads", S.solver_threads);
        count("fmm_depth", S.fmm_depth);
    }
}

}  // namespace

Settings::Settings() {
    // defaults of src/default-settings.yml
    evol_columns = {"t", "<Mx>", "<My>", "<Mz>", "E_ex", "E_demag", "E_zeeman", "E_tot"};
    vol_default.name = "__default__";
    surf_default.name = "__default__";
}

void Settings::finish() {
    if (sim_name.empty() && !mesh_file.empty()) {
        sim_name = mesh_file;
        const size_t p = sim_name.rfind('/');
        if (p != std::string::npos) sim_name.erase(0, p + 1);
        const size_t d = sim_name.rfind('.');
        if (d != std::string::npos) sim_name.erase(d);
    }
    if (mesh_file.empty()) throw SettingsError("mesh.filename is missing");
    if (vol.empty()) throw SettingsError("mesh.volume_regions is empty");
}

Settings read_settings_text(const std::string &text) {
    Settings S;
    apply_yaml(S, yaml_parse(text));
    S.finish();
    return S;
}

Settings read_settings_file(const std::string &path) {
    std::string text;
    if (path == "-") {
        std::ostringstream ss;
        ss << std::cin.rdbuf();
        text = ss.str();
    } else {
        std::ifstream in(path);
        if (!in) throw SettingsError("cannot open settings file " + path);
        std::ostringstream ss;
        ss << in.rdbuf();
        text = ss.str();
    }
    return read_settings_text(text);
}

}  // namespace fgh
