// Reader for the .oso text that oslc emits (grammar: src/liboslexec/osogram.y,
// tokens: src/liboslexec/osolex.l; sample: testsuite/unknown-instruction/test.oso).
// Hand-written (no bison/flex): one line is one header, symbol, code label or
// instruction.
#include <cctype>
#include <cstdlib>
#include <set>
#include <sstream>

#include "oslg_host.h"

namespace oslg {

std::string TypeSpec::str() const {
    std::string s;
    switch (base) {
    case BT_INT: s = "int"; break;
    case BT_FLOAT: s = "float"; break;
    case BT_TRIPLE:
        s = vecsem == VS_POINT ? "point" : vecsem == VS_NORMAL ? "normal" : vecsem == VS_COLOR ? "color" : "vector";
        break;
    case BT_MATRIX: s = "matrix"; break;
    case BT_STRING: s = "string"; break;
    case BT_CLOSURE: s = "closure color"; break;
    default: s = "void";
    }
    if (arraylen > 0) s += "[" + std::to_string(arraylen) + "]";
    if (arraylen < 0) s += "[]";
    return s;
}

static bool base_of(const std::string& t, TypeSpec& ts) {
    if (t == "int") { ts.base = BT_INT; return true; }
    if (t == "float") { ts.base = BT_FLOAT; return true; }
    if (t == "point") { ts.base = BT_TRIPLE; ts.vecsem = VS_POINT; return true; }
    if (t == "vector") { ts.base = BT_TRIPLE; ts.vecsem = VS_VECTOR; return true; }
    if (t == "normal") { ts.base = BT_TRIPLE; ts.vecsem = VS_NORMAL; return true; }
    if (t == "color") { ts.base = BT_TRIPLE; ts.vecsem = VS_COLOR; return true; }
    if (t == "matrix") { ts.base = BT_MATRIX; return true; }
    if (t == "string") { ts.base = BT_STRING; return true; }
    if (t == "void") { ts.base = BT_VOID; return true; }
    return false;
}

// "float", "color[8]", "closure color", "closure color[2]"
bool parse_typespec(const std::string& tok1, const std::string& tok2, TypeSpec& ts, int& consumed) {
    ts = TypeSpec();
    std::string t = tok1;
    consumed = 1;
    bool closure = false;
    if (t == "closure") {
        closure = true;
        t = tok2;
        consumed = 2;
    }
    std::string base = t, arr;
    size_t lb = t.find('[');
    if (lb != std::string::npos) {
        base = t.substr(0, lb);
        arr = t.substr(lb + 1, t.size() - lb - 2);
    }
    if (closure) {
        ts.base = BT_CLOSURE;
    } else if (!base_of(base, ts)) {
        return false;
    }
    if (lb != std::string::npos) ts.arraylen = arr.empty() ? -1 : std::atoi(arr.c_str());
    return true;
}

int ShaderMaster::find_symbol(const std::string& n) const {
    for (size_t i = 0; i < symbols.size(); ++i)
        if (symbols[i].name == n) return (int)i;
    return -1;
}

namespace {

// Split a line into tokens; quoted strings stay one token (quotes kept),
// "%hint{...}" stays one token even with spaces or quotes inside.
std::vector<std::string> tokenize(const std::string& line) {
    std::vector<std::string> out;
    size_t i = 0, n = line.size();
    while (i < n) {
        while (i < n && std::isspace((unsigned char)line[i])) ++i;
        if (i >= n) break;
        if (line[i] == '#') break;  // comment to end of line
        size_t start = i;
        if (line[i] == '"') {
            ++i;
            while (i < n && line[i] != '"') {
                if (line[i] == '\\' && i + 1 < n) ++i;
                ++i;
            }
            ++i;
            out.push_back(line.substr(start, i - start));
            continue;
        }
        int depth = 0;
        bool inq = false;
        while (i < n) {
            char c = line[i];
            if (inq) {
                if (c == '\\' && i + 1 < n) ++i;
                else if (c == '"') inq = false;
            } else if (c == '"') {
                inq = true;
            } else if (c == '{') {
                ++depth;
            } else if (c == '}') {
                --depth;
            } else if (std::isspace((unsigned char)c) && depth <= 0) {
                break;
            }
            ++i;
        }
        out.push_back(line.substr(start, i - start));
    }
    return out;
}

bool is_number(const std::string& s) {
    if (s.empty()) return false;
    char* end = nullptr;
    std::strtod(s.c_str(), &end);
    return end && *end == 0;
}

bool is_int(const std::string& s) {
    if (s.empty()) return false;
    size_t i = (s[0] == '-' || s[0] == '+') ? 1 : 0;
    if (i >= s.size()) return false;
    for (; i < s.size(); ++i)
        if (!std::isdigit((unsigned char)s[i])) return false;
    return true;
}

std::string unquote(const std::string& s) {
    if (s.size() >= 2 && s.front() == '"' && s.back() == '"') {
        std::string r;
        for (size_t i = 1; i + 1 < s.size(); ++i) {
            if (s[i] == '\\' && i + 2 < s.size()) {
                ++i;
                r.push_back(s[i] == 'n' ? '\n' : s[i] == 't' ? '\t' : s[i]);
            } else {
                r.push_back(s[i]);
            }
        }
        return r;
    }
    return s;
}

// The instruction names a .oso may use: the reference's op descriptor
// table (src/liboslexec/shadingsys.cpp:1300-1466, setup_op_descriptors).
// An instruction outside it is refused while parsing, as
// OSOReaderToMaster::instruction does (src/liboslexec/loadshader.cpp:500-510);
// ops this executor cannot lower are refused later, when a group is lowered.
bool known_instruction(const std::string& n) {
    static const std::set<std::string> ops = {
        "aassign", "abs", "acos", "add", "and", "area", "aref", "arraycopy", "arraylength", "asin",
        "assign", "atan", "atan2", "backfacing", "bitand", "bitor", "blackbody", "break",
        "calculatenormal", "cbrt", "ceil", "cellnoise", "clamp", "closure", "color", "compassign",
        "compl", "compref", "concat", "continue", "cos", "cosh", "cross", "degrees", "determinant",
        "dict_find", "dict_next", "dict_value", "distance", "div", "dot", "Dx", "Dy", "Dz", "dowhile",
        "end", "endswith", "environment", "eq", "erf", "erfc", "error", "exit", "exp", "exp2", "expm1",
        "fabs", "filterwidth", "floor", "fmod", "for", "format", "fprintf", "functioncall",
        "functioncall_nr", "ge", "getattribute", "getchar", "getmatrix", "getmessage",
        "gettextureinfo", "gt", "hash", "hashnoise", "if", "inversesqrt", "isconnected",
        "isconstant", "isfinite", "isinf", "isnan", "le", "length", "log", "log10", "log2", "logb",
        "lt", "luminance", "matrix", "max", "mxcompassign", "mxcompref", "min", "mix", "mod", "mul",
        "neg", "neq", "noise", "nop", "normal", "normalize", "or", "pnoise", "point",
        "pointcloud_search", "pointcloud_get", "pointcloud_write", "pow", "printf", "psnoise",
        "radians", "raytype", "regex_match", "regex_search", "return", "round", "select",
        "setmessage", "shl", "shr", "sign", "sin", "sincos", "sinh", "smoothstep", "snoise",
        "spline", "splineinverse", "split", "sqrt", "startswith", "step", "stof", "stoi", "strlen",
        "strtof", "strtoi", "sub", "substr", "surfacearea", "tan", "tanh", "texture", "texture3d",
        "trace", "transform", "transformc", "transformn", "transformv", "transpose", "trunc",
        "useparam", "vector", "warning", "wavelength_color", "while", "xor" };
    return ops.count(n) != 0;
}

}  // namespace

bool parse_oso(const std::string& text, ShaderMaster& m, std::string& err) {
    std::istringstream in(text);
    std::string line;
    int lineno = 0;
    bool in_code = false;
    std::string codelabel;
    std::vector<std::vector<std::string>> pending_ops;  // resolved after all symbols
    std::vector<int> pending_lines;
    std::vector<std::string> labels_at;                 // label for op index
    std::map<std::string, int> label_start;
    std::vector<std::pair<std::string, int>> label_order;

    while (std::getline(in, line)) {
        ++lineno;
        std::vector<std::string> tok = tokenize(line);
        if (tok.empty()) continue;
        const std::string& t0 = tok[0];
        if (t0 == "OpenShadingLanguage") continue;
        if (!in_code && (t0 == "shader" || t0 == "surface" || t0 == "displacement" || t0 == "volume"
                         || t0 == "light")) {
            if (tok.size() < 2) { err = "missing shader name"; return false; }
            m.shadertype = t0;
            m.name = tok[1];
            continue;
        }
        if (t0 == "code") {
            in_code = true;
            codelabel = tok.size() > 1 ? tok[1] : "___main___";
            label_start[codelabel] = (int)pending_ops.size();
            label_order.push_back({ codelabel, (int)pending_ops.size() });
            continue;
        }
        if (!in_code) {
            SymKind kind;
            if (t0 == "param") kind = SK_PARAM;
            else if (t0 == "oparam") kind = SK_OPARAM;
            else if (t0 == "global") kind = SK_GLOBAL;
            else if (t0 == "local") kind = SK_LOCAL;
            else if (t0 == "temp") kind = SK_TEMP;
            else if (t0 == "const") kind = SK_CONST;
            else { err = "line " + std::to_string(lineno) + ": unknown symbol kind '" + t0 + "'"; return false; }
            if (tok.size() < 3) { err = "line " + std::to_string(lineno) + ": short symbol line"; return false; }
            Symbol s;
            s.kind = kind;
            int used = 0;
            if (!parse_typespec(tok[1], tok.size() > 2 ? tok[2] : "", s.type, used)) {
                err = "line " + std::to_string(lineno) + ": bad type '" + tok[1] + "'";
                return false;
            }
            size_t i = 1 + used;
            if (i >= tok.size()) { err = "line " + std::to_string(lineno) + ": missing name"; return false; }
            s.name = tok[i++];
            for (; i < tok.size(); ++i) {
                const std::string& t = tok[i];
                if (t[0] == '%') {
                    if (t.rfind("%meta{", 0) == 0 && t.find("lockgeom") != std::string::npos) {
                        size_t c = t.rfind(',');
                        if (c != std::string::npos) s.lockgeom = std::atoi(t.c_str() + c + 1) != 0;
                    } else if (t == "%initexpr") {
                        s.has_init_ops = true;
                    }
                    continue;
                }
                if (t[0] == '"') s.sdefault.push_back(unquote(t));
                else if (is_number(t)) s.fdefault.push_back((float)std::strtod(t.c_str(), nullptr));
            }
            if (m.find_symbol(s.name) >= 0) { err = "duplicate symbol " + s.name; return false; }
            m.symbols.push_back(s);
            continue;
        }
        // instruction
        if (t0 == "end" && tok.size() == 1) {
            // "end" closes the code body; record it as an op like oslc does
            pending_ops.push_back({ "end" });
            pending_lines.push_back(lineno);
            continue;
        }
        pending_ops.push_back(tok);
        pending_lines.push_back(lineno);
    }

    // resolve ops
    for (size_t k = 0; k < pending_ops.size(); ++k) {
        const std::vector<std::string>& tok = pending_ops[k];
        if (!known_instruction(tok[0])) {
            err = "Parsing shader \"" + m.name + "\": instruction \"" + tok[0]
                + "\" is not known. Maybe compiled with a too-new oslc?";
            return false;
        }
        OsoOp op;
        op.name = tok[0];
        op.line = pending_lines[k];
        for (size_t i = 1; i < tok.size(); ++i) {
            const std::string& t = tok[i];
            if (t[0] == '%') {
                if (t.rfind("%argrw{", 0) == 0) op.argrw = unquote(t.substr(7, t.size() - 8));
                continue;
            }
            if (is_int(t) && m.find_symbol(t) < 0) {
                op.jumps.push_back(std::atoi(t.c_str()));
                continue;
            }
            int si = m.find_symbol(t);
            if (si < 0) {
                err = "line " + std::to_string(op.line) + ": unknown symbol '" + t + "' in op " + op.name;
                return false;
            }
            op.args.push_back(si);
        }
        m.ops.push_back(op);
    }
    // code sections: ___main___ and per-param init code
    for (size_t li = 0; li < label_order.size(); ++li) {
        int b = label_order[li].second;
        int e = li + 1 < label_order.size() ? label_order[li + 1].second : (int)m.ops.size();
        const std::string& lab = label_order[li].first;
        if (lab == "___main___") {
            m.maincodebegin = b;
            m.maincodeend = e;
        } else {
            int si = m.find_symbol(lab);
            if (si >= 0) {
                m.symbols[si].has_init_ops = true;
                m.symbols[si].initbegin = b;
                m.symbols[si].initend = e;
            }
        }
    }
    if (label_order.empty()) {
        m.maincodebegin = 0;
        m.maincodeend = (int)m.ops.size();
    }
    if (m.name.empty()) { err = "no shader declaration"; return false; }
    return true;
}

}  // namespace oslg
