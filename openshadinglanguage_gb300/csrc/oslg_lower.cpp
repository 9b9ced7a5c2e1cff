// Lowering of an optimized ShaderGroup into the device op program.
//
// What the reference does at this point is JIT the group: BatchedAnalysis
// (src/liboslexec/batched_analysis.cpp:1326, :2882) decides which symbols
// are varying and how control flow is masked, the RuntimeOptimizer marks
// which symbols carry derivatives (runtimeoptimize.cpp:3218-3234), and
// BatchedBackendLLVM lays out the SoA groupdata heap
// (batched_llvm_instance.cpp:918-1054) and emits one masked function per
// layer. Here the same decisions are made once on the host and written out
// as a compact op stream:
//   * derivative marking: a symbol carries [val,dx,dy] if a renderer output
//     asks for derivatives or a deriv-consuming op (Dx/Dy/area/filterwidth)
//     reads it, propagated backwards through every op whose result
//     derivatives depend on its inputs;
//   * constant pooling: const symbols and parameters that no op writes and
//     nothing binds (no connection, no userdata) are uniform values;
//   * layout: everything else gets heap slots ([val][dx][dy] blocks);
//   * control flow: if/loops become mask ops (OP_IF/ELSE/ENDIF, OP_LOOP_*).
//   * dead ops: an op survives only if it has an effect outside the symbol
//     heap (stores, BSDF output, control flow, messages) or writes a symbol
//     a surviving op reads (the RuntimeOptimizer's dead-code removal,
//     runtimeoptimize.cpp:2133-2186, done flow-insensitively here so that
//     loops need no special case).
//   * layers run in group order; a connection copies the upstream output
//     into the downstream parameter before that layer's body.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <set>
#include <sstream>

#include "oslg_host.h"

namespace oslg {

namespace {

struct GSym {
    int layer = -1;
    std::string name;
    TypeSpec type;
    SymKind kind = SK_LOCAL;
    bool derivs = false;
    bool is_const = false;
    std::vector<float> cval;
    std::vector<std::string> sval;
    int global_id = -1;
    int slot = -1;
    bool written = false;
    bool referenced = false;
};

struct LOp {
    std::string name;
    std::vector<int> args;   // gsym indices
    std::vector<int> jumps;  // LOp indices
    int layer = -1;
    bool param_init = false;     // assign that sets a parameter to its value
    int param_gsym = -1;
    int64_t imm[4] = { 0, 0, 0, 0 };
    std::string argrw;
};

const char* kGlobalNames[G_COUNT] = { "P", "dPdx", "dPdy", "dPdz", "I", "dIdx", "dIdy", "N", "Ng",
                                      "u", "dudx", "dudy", "v", "dvdx", "dvdy", "dPdu", "dPdv",
                                      "time", "dtime", "dPdtime", "Ps", "dPsdx", "dPsdy",
                                      "surfacearea", "$flipHandedness", "$backfacing" };

int global_id_of(const std::string& n) {
    for (int i = 0; i < (int)G_COUNT; ++i)
        if (n == kGlobalNames[i]) return i;
    return -1;
}

// Globals whose derivatives the caller supplies (dPdx/dPdy style fields).
bool global_has_derivs(int gid) {
    return gid == G_P || gid == G_I || gid == G_U || gid == G_V || gid == G_PS;
}

uint32_t string_hash(const std::string& s) {
    // FNV-1a: strings only need stable equality on the device
    uint32_t h = 2166136261u;
    for (unsigned char c : s) { h ^= c; h *= 16777619u; }
    return h;
}

// CIE 1931 2-degree colour matching functions (x-bar, y-bar, z-bar) at 5 nm
// from 380 to 780 nm, four decimals: the published CIE data the reference's
// blackbody integrates against (src/liboslexec/opcolor_impl.h:55-93).
const float kCIE[81][3] = {
    { 0.0014f, 0.0000f, 0.0065f },  // 380 nm
    { 0.0022f, 0.0001f, 0.0105f },  // 385 nm
    { 0.0042f, 0.0001f, 0.0201f },  // 390 nm
    { 0.0076f, 0.0002f, 0.0362f },  // 395 nm
    { 0.0143f, 0.0004f, 0.0679f },  // 400 nm
    { 0.0232f, 0.0006f, 0.1102f },  // 405 nm
    { 0.0435f, 0.0012f, 0.2074f },  // 410 nm
    { 0.0776f, 0.0022f, 0.3713f },  // 415 nm
    { 0.1344f, 0.0040f, 0.6456f },  // 420 nm
    { 0.2148f, 0.0073f, 1.0391f },  // 425 nm
    { 0.2839f, 0.0116f, 1.3856f },  // 430 nm
    { 0.3285f, 0.0168f, 1.6230f },  // 435 nm
    { 0.3483f, 0.0230f, 1.7471f },  // 440 nm
    { 0.3481f, 0.0298f, 1.7826f },  // 445 nm
    { 0.3362f, 0.0380f, 1.7721f },  // 450 nm
    { 0.3187f, 0.0480f, 1.7441f },  // 455 nm
    { 0.2908f, 0.0600f, 1.6692f },  // 460 nm
    { 0.2511f, 0.0739f, 1.5281f },  // 465 nm
    { 0.1954f, 0.0910f, 1.2876f },  // 470 nm
    { 0.1421f, 0.1126f, 1.0419f },  // 475 nm
    { 0.0956f, 0.1390f, 0.8130f },  // 480 nm
    { 0.0580f, 0.1693f, 0.6162f },  // 485 nm
    { 0.0320f, 0.2080f, 0.4652f },  // 490 nm
    { 0.0147f, 0.2586f, 0.3533f },  // 495 nm
    { 0.0049f, 0.3230f, 0.2720f },  // 500 nm
    { 0.0024f, 0.4073f, 0.2123f },  // 505 nm
    { 0.0093f, 0.5030f, 0.1582f },  // 510 nm
    { 0.0291f, 0.6082f, 0.1117f },  // 515 nm
    { 0.0633f, 0.7100f, 0.0782f },  // 520 nm
    { 0.1096f, 0.7932f, 0.0573f },  // 525 nm
    { 0.1655f, 0.8620f, 0.0422f },  // 530 nm
    { 0.2257f, 0.9149f, 0.0298f },  // 535 nm
    { 0.2904f, 0.9540f, 0.0203f },  // 540 nm
    { 0.3597f, 0.9803f, 0.0134f },  // 545 nm
    { 0.4334f, 0.9950f, 0.0087f },  // 550 nm
    { 0.5121f, 1.0000f, 0.0057f },  // 555 nm
    { 0.5945f, 0.9950f, 0.0039f },  // 560 nm
    { 0.6784f, 0.9786f, 0.0027f },  // 565 nm
    { 0.7621f, 0.9520f, 0.0021f },  // 570 nm
    { 0.8425f, 0.9154f, 0.0018f },  // 575 nm
    { 0.9163f, 0.8700f, 0.0017f },  // 580 nm
    { 0.9786f, 0.8163f, 0.0014f },  // 585 nm
    { 1.0263f, 0.7570f, 0.0011f },  // 590 nm
    { 1.0567f, 0.6949f, 0.0010f },  // 595 nm
    { 1.0622f, 0.6310f, 0.0008f },  // 600 nm
    { 1.0456f, 0.5668f, 0.0006f },  // 605 nm
    { 1.0026f, 0.5030f, 0.0003f },  // 610 nm
    { 0.9384f, 0.4412f, 0.0002f },  // 615 nm
    { 0.8544f, 0.3810f, 0.0002f },  // 620 nm
    { 0.7514f, 0.3210f, 0.0001f },  // 625 nm
    { 0.6424f, 0.2650f, 0.0000f },  // 630 nm
    { 0.5419f, 0.2170f, 0.0000f },  // 635 nm
    { 0.4479f, 0.1750f, 0.0000f },  // 640 nm
    { 0.3608f, 0.1382f, 0.0000f },  // 645 nm
    { 0.2835f, 0.1070f, 0.0000f },  // 650 nm
    { 0.2187f, 0.0816f, 0.0000f },  // 655 nm
    { 0.1649f, 0.0610f, 0.0000f },  // 660 nm
    { 0.1212f, 0.0446f, 0.0000f },  // 665 nm
    { 0.0874f, 0.0320f, 0.0000f },  // 670 nm
    { 0.0636f, 0.0232f, 0.0000f },  // 675 nm
    { 0.0468f, 0.0170f, 0.0000f },  // 680 nm
    { 0.0329f, 0.0119f, 0.0000f },  // 685 nm
    { 0.0227f, 0.0082f, 0.0000f },  // 690 nm
    { 0.0158f, 0.0057f, 0.0000f },  // 695 nm
    { 0.0114f, 0.0041f, 0.0000f },  // 700 nm
    { 0.0081f, 0.0029f, 0.0000f },  // 705 nm
    { 0.0058f, 0.0021f, 0.0000f },  // 710 nm
    { 0.0041f, 0.0015f, 0.0000f },  // 715 nm
    { 0.0029f, 0.0010f, 0.0000f },  // 720 nm
    { 0.0020f, 0.0007f, 0.0000f },  // 725 nm
    { 0.0014f, 0.0005f, 0.0000f },  // 730 nm
    { 0.0010f, 0.0004f, 0.0000f },  // 735 nm
    { 0.0007f, 0.0002f, 0.0000f },  // 740 nm
    { 0.0005f, 0.0002f, 0.0000f },  // 745 nm
    { 0.0003f, 0.0001f, 0.0000f },  // 750 nm
    { 0.0002f, 0.0001f, 0.0000f },  // 755 nm
    { 0.0002f, 0.0001f, 0.0000f },  // 760 nm
    { 0.0001f, 0.0000f, 0.0000f },  // 765 nm
    { 0.0001f, 0.0000f, 0.0000f },  // 770 nm
    { 0.0001f, 0.0000f, 0.0000f },  // 775 nm
    { 0.0000f, 0.0000f, 0.0000f },  // 780 nm
};

// Ops whose result derivatives are a function of their inputs' derivatives.
const std::set<std::string>& deriv_propagating_ops() {
    static const std::set<std::string> s = {
        "assign", "add", "sub", "mul", "div", "neg", "compref", "compassign", "point", "vector",
        "normal", "color", "aref", "aassign", "sin", "cos", "tan", "asin", "acos", "atan", "atan2",
        "sinh", "cosh", "tanh", "exp", "exp2", "expm1", "log", "log2", "log10", "pow", "sqrt",
        "inversesqrt", "cbrt", "abs", "fabs", "mix", "clamp", "min", "max", "smoothstep", "select",
        "dot", "cross", "length", "normalize", "distance", "transform", "transformv", "transformn",
        "noise", "snoise", "pnoise", "psnoise", "spline", "splineinverse", "mod", "fmod", "luminance", "radians",
        "transformc", "sincos", "arraycopy",
        "degrees", "erf", "erfc" };
    return s;
}

struct Lowerer {
    ShadingSystem& ss;
    ShaderGroup& g;
    std::string& err;
    std::vector<GSym> syms;
    std::vector<LOp> lops;
    std::map<std::pair<int, int>, int> layer_sym;  // (layer, master sym) -> gsym
    std::map<std::string, int> globals;
    // outputs
    std::vector<Op> ops;
    std::vector<std::string> op_names;
    std::vector<uint32_t> pool;  // constant pool words
    uint32_t heap_top = 0;
    uint32_t max_depth = 0;
    std::vector<int> fret_ops;  // emitted OP_FUNC_RETURN ops (their end pc is patched)
    bool uses_closures = false;
    bool wide_nodes = false;  // some closure fills more than kRecordParams parameter words
    // messages: per name a state symbol, per (name, type) a value store
    std::map<std::string, int> msg_state;
    std::map<std::string, int> msg_store;
    std::map<std::string, int> msg_type_id;

    int stop_layer = -1;  // >= 0: run layers [0, stop_layer] only (execute_layer)

    Lowerer(ShadingSystem& s, ShaderGroup& gg, std::string& e) : ss(s), g(gg), err(e) {}
    int last_layer() const { return stop_layer >= 0 ? stop_layer : (int)g.layers.size() - 1; }

    bool fail(const std::string& m) { err = m; return false; }

    int add_sym(const GSym& s) { syms.push_back(s); return (int)syms.size() - 1; }

    int const_float(float v) {
        GSym s; s.name = "$c"; s.type.base = BT_FLOAT; s.kind = SK_CONST; s.is_const = true;
        s.cval = { v };
        return add_sym(s);
    }
    int const_int(int v) {
        GSym s; s.name = "$ci"; s.type.base = BT_INT; s.kind = SK_CONST; s.is_const = true;
        s.cval = { (float)v };
        return add_sym(s);
    }

    int global_sym(const std::string& name, const TypeSpec& ts) {
        auto it = globals.find(name);
        if (it != globals.end()) return it->second;
        GSym s;
        s.name = name; s.type = ts; s.kind = SK_GLOBAL; s.global_id = global_id_of(name);
        int id = add_sym(s);
        globals[name] = id;
        return id;
    }

    // gsym for master symbol `msi` of layer `li`
    int sym_of(int li, int msi) {
        auto key = std::make_pair(li, msi);
        auto it = layer_sym.find(key);
        if (it != layer_sym.end()) return it->second;
        const Symbol& ms = g.layers[li].master->symbols[msi];
        int id;
        if (ms.kind == SK_GLOBAL) {
            id = global_sym(ms.name, ms.type);
        } else {
            GSym s;
            s.layer = li; s.name = ms.name; s.type = ms.type; s.kind = ms.kind;
            if (ms.kind == SK_CONST) {
                s.is_const = true;
                s.cval = ms.fdefault;
                s.sval = ms.sdefault;
            }
            id = add_sym(s);
        }
        layer_sym[key] = id;
        return id;
    }

    const SymLoc* find_symloc(int li, const std::string& name, SymArena arena) {
        const std::string& lname = g.layers[li].layername;
        for (const SymLoc& sl : g.symlocs) {
            if (sl.arena != arena) continue;
            if (sl.name == lname + "." + name) return &sl;
        }
        for (const SymLoc& sl : g.symlocs) {
            if (sl.arena != arena) continue;
            if (sl.name == name) return &sl;
        }
        return nullptr;
    }

    // Copy master ops [b,e) of layer li into lops, remapping jumps.
    void copy_section(int li, int b, int e) {
        const ShaderMaster& m = *g.layers[li].master;
        int base = (int)lops.size();
        for (int k = b; k < e; ++k) {
            const OsoOp& mo = m.ops[k];
            LOp op;
            op.name = mo.name;
            op.layer = li;
            op.argrw = mo.argrw;
            for (int a : mo.args) op.args.push_back(sym_of(li, a));
            for (int j : mo.jumps) op.jumps.push_back(base + (j - b));
            if (op.name == "end") op.name = "nop";
            lops.push_back(op);
        }
    }

    bool build_lops() {
        for (int li = 0; li <= last_layer(); ++li) {
            Layer& L = g.layers[li];
            const ShaderMaster& m = *L.master;
            for (int msi = 0; msi < (int)m.symbols.size(); ++msi) {
                const Symbol& ms = m.symbols[msi];
                if (ms.kind != SK_PARAM && ms.kind != SK_OPARAM) continue;
                int gs = sym_of(li, msi);
                // 1. connection into this parameter
                const Connection* conn = nullptr;
                for (const Connection& c : L.connections)
                    if (c.dstparam == ms.name) conn = &c;
                if (conn) {
                    int srcm = g.layers[conn->srclayer].master->find_symbol(conn->srcparam);
                    if (srcm < 0)
                        return fail("connection source " + conn->srcparam + " not found in layer "
                                    + g.layers[conn->srclayer].layername);
                    int src = sym_of(conn->srclayer, srcm);
                    LOp op; op.name = "assign"; op.layer = li; op.args = { gs, src };
                    lops.push_back(op);
                    continue;
                }
                // instance value / lockgeom
                const InstanceParam* ip = nullptr;
                for (const InstanceParam& p : L.params)
                    if (p.name == ms.name) ip = &p;
                bool lockgeom = ip ? ip->lockgeom : ms.lockgeom;
                // 2. userdata binding for varying (lockgeom=0) parameters
                if (!lockgeom) {
                    const SymLoc* sl = find_symloc(li, ms.name, ARENA_USERDATA);
                    if (sl) {
                        LOp op; op.name = "__load_userdata"; op.layer = li; op.args = { gs };
                        op.imm[0] = sl->offset; op.imm[1] = sl->stride;
                        op.imm[2] = sl->derivs ? 1 : 0;
                        lops.push_back(op);
                        continue;
                    }
                }
                // 3. explicit instance value
                if (ip) {
                    GSym c; c.name = "$pv"; c.type = ms.type; c.kind = SK_CONST; c.is_const = true;
                    c.cval = ip->fvals; c.sval = ip->svals;
                    int cs = add_sym(c);
                    LOp op; op.name = "assign"; op.layer = li; op.args = { gs, cs };
                    op.param_init = lockgeom; op.param_gsym = gs;
                    lops.push_back(op);
                    continue;
                }
                // 4. default-value code
                if (ms.has_init_ops && ms.initend > ms.initbegin) {
                    copy_section(li, ms.initbegin, ms.initend);
                    continue;
                }
                // 5. plain default
                GSym c; c.name = "$pd"; c.type = ms.type; c.kind = SK_CONST; c.is_const = true;
                c.cval = ms.fdefault; c.sval = ms.sdefault;
                int cs = add_sym(c);
                LOp op; op.name = "assign"; op.layer = li; op.args = { gs, cs };
                op.param_init = lockgeom; op.param_gsym = gs;
                lops.push_back(op);
            }
            copy_section(li, m.maincodebegin, m.maincodeend);
            LOp le; le.name = "__layer_end"; le.layer = li;
            lops.push_back(le);
            // the layer's outputs are final here: stored for every point that
            // ran the layer, including those that exited inside it
            if (!push_stores(li)) return false;
            LOp se; se.name = "__stores_end"; se.layer = li;
            lops.push_back(se);
        }
        // renderer-side work and stores of globals, for every point
        LOp fin; fin.name = "__stores_end"; fin.imm[0] = 1;
        lops.push_back(fin);
        // renderer-side BSDF evaluation of closure outputs
        for (const BsdfEvalRequest& be : g.bsdf_evals) {
            SymLoc tmp;
            tmp.name = be.closure;
            if (beyond_stop(be.closure)) continue;
            int gs = resolve_symloc(tmp);
            if (gs < 0 || syms[gs].type.base != BT_CLOSURE)
                return fail("bsdf eval: '" + be.closure + "' is not a closure of the group");
            GSym d; d.name = "$wi"; d.type.base = BT_TRIPLE; d.type.vecsem = VS_VECTOR; d.kind = SK_CONST;
            d.is_const = true; d.cval = { be.wi[0], be.wi[1], be.wi[2] };
            int wi = add_sym(d);
            TypeSpec vt; vt.base = BT_TRIPLE; vt.vecsem = VS_VECTOR;
            int I = global_sym("I", vt);
            LOp op; op.name = "__bsdf_eval"; op.args = { gs, wi, I };
            op.imm[0] = be.offset; op.imm[1] = be.stride;
            lops.push_back(op);
        }
        for (const BsdfSampleRequest& bs : g.bsdf_samples) {
            SymLoc tmp;
            tmp.name = bs.closure;
            if (beyond_stop(bs.closure)) continue;
            int gs = resolve_symloc(tmp);
            if (gs < 0 || syms[gs].type.base != BT_CLOSURE)
                return fail("bsdf sample: '" + bs.closure + "' is not a closure of the group");
            TypeSpec vt; vt.base = BT_TRIPLE; vt.vecsem = VS_VECTOR;
            int I = global_sym("I", vt);
            LOp op; op.name = "__bsdf_sample"; op.args = { gs, I };
            op.imm[0] = bs.offset; op.imm[1] = bs.stride; op.imm[2] = bs.in_offset; op.imm[3] = bs.in_stride;
            lops.push_back(op);
        }
        return push_stores(-1);
    }

    // Stores of the renderer outputs placed through symlocs whose symbol
    // belongs to layer li (-1: shader globals), in symloc order.
    bool push_stores(int li) {
        for (const SymLoc& sl : g.symlocs) {
            if (sl.arena != ARENA_OUTPUTS) continue;
            if (beyond_stop(sl.name)) continue;  // written by a layer that does not run
            int gs = resolve_symloc(sl);
            if (gs < 0) return fail("symloc '" + sl.name + "' does not name a symbol of the group");
            if (syms[gs].layer != li) continue;
            LOp op; op.name = "__store_output"; op.args = { gs };
            op.imm[0] = sl.offset; op.imm[1] = sl.stride; op.imm[2] = sl.derivs ? 1 : 0;
            op.imm[3] = sl.type.arraylen > 0 ? sl.type.arraylen : 4;  // closure records kept
            lops.push_back(op);
        }
        for (const auto& r : g.retained) {  // find_symbol's symbols of this layer
            if (r->layer != li || li < 0 || (stop_layer >= 0 && li > stop_layer)) continue;
            const int msi = g.layers[(size_t)li].master->find_symbol(r->name);
            if (msi < 0) return fail("retained symbol '" + r->name + "' is not in its layer");
            LOp op; op.name = "__store_heap"; op.args = { sym_of(li, msi) };
            op.imm[0] = r->plane; op.imm[1] = r->words;
            lops.push_back(op);
        }
        return true;
    }

    // a "layer.symbol" name of a layer past the stop layer
    bool beyond_stop(const std::string& name) const {
        const size_t dot = name.find('.');
        if (dot == std::string::npos) return false;
        return g.find_layer(name.substr(0, dot)) > last_layer();
    }
    int resolve_symloc(const SymLoc& sl) {
        std::string lname, sname = sl.name;
        size_t dot = sl.name.find('.');
        if (dot != std::string::npos) {
            lname = sl.name.substr(0, dot);
            sname = sl.name.substr(dot + 1);
        }
        for (int li = (int)g.layers.size() - 1; li >= 0; --li) {
            if (!lname.empty() && g.layers[li].layername != lname) continue;
            if (lname.empty() && li > last_layer()) continue;
            int msi = g.layers[li].master->find_symbol(sname);
            if (msi >= 0) return sym_of(li, msi);
        }
        return -1;
    }

    // ---- analysis ----------------------------------------------------------
    static bool writes_arg(const LOp& op, int i) {
        // after prepare_messages: setmessage (name, value, state, store),
        // getmessage (result, name, dest, state, store)
        if (op.name == "setmessage") return i == 2 || i == 3;
        if (op.name == "getmessage") return i == 0 || i == 2 || i == 3;
        if (op.name == "getattribute" || op.name == "gettextureinfo") return i == 0 || i == (int)op.args.size() - 1;
        if (op.name == "getmatrix") return i == 0 || i == 3;
        if (!op.argrw.empty() && i < (int)op.argrw.size())
            return op.argrw[i] == 'w' || op.argrw[i] == 'W';
        static const std::set<std::string> nowrite = {
            "if", "for", "while", "dowhile", "break", "continue", "return", "exit", "nop",
            "useparam", "__layer_end", "__store_output", "__bsdf_eval", "__bsdf_sample", "__cl_store",
            "__cl_bsdf_eval", "__cl_bsdf_sample", "functioncall",
            "functioncall_nr", "__fret", "__stores_end", "__store_heap",
            "printf", "warning", "error", "fprintf" };
        if (nowrite.count(op.name)) return false;
        if (op.name == "sincos") return i == 1 || i == 2;
        return i == 0;
    }

    void analyze() {
        for (const LOp& op : lops) {
            if (op.param_init) continue;
            for (size_t i = 0; i < op.args.size(); ++i)
                if (writes_arg(op, (int)i)) syms[op.args[i]].written = true;
        }
        // parameters nobody writes and nothing binds become uniform constants
        for (LOp& op : lops) {
            if (!op.param_init) continue;
            GSym& p = syms[op.param_gsym];
            if (!p.written && p.type.base != BT_CLOSURE) {
                const GSym& c = syms[op.args[1]];
                p.is_const = true;
                p.cval = c.cval;
                p.sval = c.sval;
                op.name = "nop";
                op.args.clear();
            }
        }
        // derivative seeds
        for (const LOp& op : lops) {
            if ((op.name == "Dx" || op.name == "Dy" || op.name == "Dz" || op.name == "area"
                 || op.name == "filterwidth" || op.name == "calculatenormal")
                && op.args.size() > 1)
                mark_derivs(op.args[1]);
            // gabor noise always takes derivatives of its positions
            // (src/liboslcomp/typecheck.cpp:1363-1378)
            if ((op.name == "noise" || op.name == "pnoise") && op.args.size() > 2 && is_string(op.args[1])
                && syms[op.args[1]].is_const && const_string(op.args[1]) == "gabor") {
                for (size_t i = 2; i < op.args.size() && !is_string(op.args[i]); ++i) mark_derivs(op.args[i]);
            }
            if (op.name == "__store_output" && op.imm[2]) mark_derivs(op.args[0]);
            // texture's footprint comes from the derivatives of s and t,
            // environment's from those of the direction
            if (op.name == "texture" && op.args.size() > 3) {
                mark_derivs(op.args[2]);
                mark_derivs(op.args[3]);
            }
            if (op.name == "environment" && op.args.size() > 2) mark_derivs(op.args[2]);
            if (op.name == "__load_userdata" && op.imm[2]) mark_derivs(op.args[0]);
        }
        const auto& prop = deriv_propagating_ops();
        bool changed = true;
        while (changed) {
            changed = false;
            for (int k = (int)lops.size() - 1; k >= 0; --k) {
                const LOp& op = lops[k];
                if (!prop.count(op.name) || op.args.empty()) continue;
                bool res_needs = false;
                for (size_t i = 0; i < op.args.size(); ++i)
                    if (writes_arg(op, (int)i) && syms[op.args[i]].derivs) res_needs = true;
                if (!res_needs) continue;
                for (size_t i = 0; i < op.args.size(); ++i) {
                    if (writes_arg(op, (int)i) && op.name != "compassign" && op.name != "aassign")
                        continue;
                    // index operands of compref/aref/compassign/aassign carry no derivs
                    if ((op.name == "compref" || op.name == "aref") && i == 2) continue;
                    if ((op.name == "compassign" || op.name == "aassign") && i == 1) continue;
                    if ((op.name == "spline" || op.name == "splineinverse") && i == 1) continue;  // basis name
                    // the knot count; splineinverse ignores knot derivatives
                    if ((op.name == "spline" || op.name == "splineinverse") && op.args.size() == 5 && i == 3) continue;
                    if (op.name == "splineinverse" && i + 1 == op.args.size()) continue;
                    if ((op.name == "noise" || op.name == "snoise" || op.name == "pnoise"
                         || op.name == "psnoise")
                        && i == 1 && syms[op.args[1]].type.base == BT_STRING)
                        continue;
                    int a = op.args[i];
                    if (!syms[a].derivs && syms[a].type.derivable() && !syms[a].is_const) {
                        syms[a].derivs = true;
                        changed = true;
                    }
                }
            }
        }
        for (GSym& s : syms)
            if (s.is_const) s.derivs = false;
    }

    // ---- messages ------------------------------------------------------------
    // setmessage/getmessage with constant names become ops on hidden
    // per-point symbols. A getmessage that no earlier setmessage of its name
    // precedes (in layer and op order) can never find a message and becomes
    // `result = 0`, as constfold_getmessage does
    // (src/liboslexec/constfold.cpp:2240-2258). A sourced getmessage asks
    // the renderer, whose default answer is "not found"
    // (batched_rendererservices.h getmessage): it folds to 0 as well.
    static std::string msg_type_key(const TypeSpec& t) {
        return std::to_string((int)t.base) + ":" + std::to_string((int)t.vecsem) + ":" + std::to_string(t.arraylen);
    }
    int msg_store_for(const std::string& name, const TypeSpec& t) {
        const std::string key = name + "|" + msg_type_key(t);
        auto it = msg_store.find(key);
        if (it != msg_store.end()) return it->second;
        GSym v; v.name = "$msg." + name; v.type = t; v.kind = SK_LOCAL;
        int id = add_sym(v);
        msg_store[key] = id;
        return id;
    }
    uint32_t msg_tid(const TypeSpec& t) {
        auto ins = msg_type_id.insert({ msg_type_key(t), (int)msg_type_id.size() });
        return (uint32_t)ins.first->second;
    }
    // A layer other than the last with no outgoing connection and no
    // renderer output is unused and removed, as ShaderInstance::unused()
    // decides with the default lazyunconnected
    // (src/liboslexec/oslexec_pvt.h:1477-1491): its messages are never sent.
    bool layer_used(int li) {
        if (li == last_layer()) return true;
        for (int lj = li + 1; lj <= last_layer(); ++lj)
            for (const Connection& c : g.layers[(size_t)lj].connections)
                if (c.srclayer == li) return true;
        auto in_layer = [&](const std::string& nm) {
            SymLoc tmp;
            tmp.name = nm;
            int gs = resolve_symloc(tmp);
            return gs >= 0 && syms[gs].layer == li;
        };
        for (const SymLoc& sl : g.symlocs)
            if (sl.arena == ARENA_OUTPUTS && in_layer(sl.name)) return true;
        for (const BsdfEvalRequest& be : g.bsdf_evals)
            if (in_layer(be.closure)) return true;
        for (const BsdfSampleRequest& bs : g.bsdf_samples)
            if (in_layer(bs.closure)) return true;
        for (const std::string& ro : g.renderer_outputs)
            if (g.layers[li].master->find_symbol(ro) >= 0) return true;
        return false;
    }
    bool prepare_messages() {
        std::set<std::string> sent;
        std::vector<int> used(g.layers.size(), -1);
        for (LOp& op : lops) {
            if (op.name == "setmessage" && op.layer >= 0) {
                if (used[op.layer] < 0) used[op.layer] = layer_used(op.layer) ? 1 : 0;
                if (!used[op.layer]) {
                    op.name = "nop";
                    op.args.clear();
                    continue;
                }
            }
            if (op.name == "setmessage") {
                if (op.args.size() != 2) return fail("setmessage takes a name and a value");
                if (!is_string(op.args[0]) || !syms[op.args[0]].is_const)
                    return fail("setmessage: the message name must be a constant string");
                const std::string nm = const_string(op.args[0]);
                if (!msg_state.count(nm)) {
                    GSym st; st.name = "$msgstate." + nm; st.type.base = BT_INT; st.kind = SK_LOCAL;
                    msg_state[nm] = add_sym(st);
                }
                const TypeSpec t = syms[op.args[1]].type;
                op.imm[0] = msg_tid(t);
                op.args = { op.args[0], op.args[1], msg_state[nm], msg_store_for(nm, t) };
                op.argrw.clear();
                sent.insert(nm);
            } else if (op.name == "getmessage") {
                const size_t na = op.args.size();
                if (na != 3 && na != 4) return fail("getmessage takes ([source,] name, value)");
                const int nsym = op.args[na - 2];
                if (!is_string(nsym) || !syms[nsym].is_const)
                    return fail("getmessage: the message name must be a constant string");
                const std::string nm = const_string(nsym);
                if (na == 4 || !sent.count(nm)) {
                    int z = const_int(0);
                    op.name = "assign";
                    op.args = { op.args[0], z };
                    op.argrw = "wr";
                    continue;
                }
                const TypeSpec t = syms[op.args[2]].type;
                op.imm[0] = msg_tid(t);
                op.args = { op.args[0], nsym, op.args[2], msg_state[nm], msg_store_for(nm, t) };
                op.argrw.clear();
            }
        }
        return true;
    }

    // ---- constant folding ------------------------------------------------------
    // Forward propagation of known values through straight-line code, as
    // the RuntimeOptimizer's constant folding and block aliases do
    // (src/liboslexec/runtimeoptimize.cpp, constfold.cpp): a symbol whose
    // last write gave it a constant value is read as that constant, and an
    // op whose inputs are all constants becomes an assignment of its
    // result. Knowledge survives an `if` only for symbols neither branch
    // writes; inside a loop nothing the loop writes is known. Folded
    // arithmetic is IEEE single precision without contraction, as the
    // kernels compute it; results that would be NaN or out of int range
    // are left to run.
    struct CVal {
        uint32_t tc = TC_FLOAT;
        int n = 1;
        uint32_t w[3] = { 0, 0, 0 };
        float f(int c) const {
            uint32_t x = w[n == 1 ? 0 : c];
            if (tc == TC_INT) return (float)(int32_t)x;
            float v;
            std::memcpy(&v, &x, 4);
            return v;
        }
        bool truth() const {
            if (tc == TC_INT) return w[0] != 0u;
            for (int c = 0; c < n; ++c)
                if (f(c) != 0.0f) return true;
            return false;
        }
    };
    static uint32_t fbits(float v) { uint32_t w; std::memcpy(&w, &v, 4); return w; }
    bool cval_of(int s, CVal& v) const {
        const GSym& g = syms[s];
        if (!g.is_const || g.type.is_array()) return false;
        if (g.type.base != BT_FLOAT && g.type.base != BT_INT && g.type.base != BT_TRIPLE) return false;
        v.n = g.type.base == BT_TRIPLE ? 3 : 1;
        v.tc = g.type.tclass();
        for (int c = 0; c < v.n; ++c) {
            if (g.slot >= 0) {  // a folded value: its pool words
                v.w[c] = pool[(size_t)g.slot + c];
                continue;
            }
            float x = g.cval.empty() ? 0.0f : g.cval[std::min<size_t>(c, g.cval.size() - 1)];
            v.w[c] = v.tc == TC_INT ? (uint32_t)(int32_t)x : fbits(x);
        }
        return true;
    }
    // the value op would compute from its (constant) operands
    bool fold_eval(const LOp& op, std::vector<uint32_t>& out) const {
        const std::string& n = op.name;
        const size_t na = op.args.size();
        if (na < 2) return false;
        const TypeSpec& rt = syms[op.args[0]].type;
        if (rt.is_array() || (rt.base != BT_FLOAT && rt.base != BT_INT && rt.base != BT_TRIPLE)) return false;
        const int nr = rt.base == BT_TRIPLE ? 3 : 1;
        const bool rint = rt.base == BT_INT;
        out.assign((size_t)nr, 0u);
        auto put = [&](int c, float v) {
            if (v != v) return false;
            if (rint) {
                if (!(v > -2147483648.0f && v < 2147483648.0f)) return false;
                out[(size_t)c] = (uint32_t)(int32_t)v;
            } else {
                out[(size_t)c] = fbits(v);
            }
            return true;
        };
        if (n == "isconstant") {
            // constfold.cpp:3030-3045: a constant here stays one; the other
            // case is decided when the op is lowered, after all folding
            if (!syms[op.args[1]].is_const) return false;
            out[0] = 1u;
            return true;
        }
        CVal x, y, z;
        const bool ctor = n == "color" || n == "point" || n == "vector" || n == "normal";
        if (n == "assign" || (ctor && na == 2)) {
            if (!cval_of(op.args[1], x) || (x.n == 3 && nr == 1)) return false;
            for (int c = 0; c < nr; ++c) {
                if (!rint && x.tc != TC_INT) out[(size_t)c] = x.w[x.n == 1 ? 0 : c];
                else if (rint && x.tc == TC_INT) out[(size_t)c] = x.w[0];
                else if (!put(c, x.f(c))) return false;
            }
            return true;
        }
        if (ctor && na == 4) {
            for (int c = 0; c < 3; ++c)
                if (!cval_of(op.args[1 + c], x) || x.n != 1 || !put(c, x.f(0))) return false;
            return nr == 3;
        }
        if (n == "neg") {
            if (!cval_of(op.args[1], x)) return false;
            if (rint) {
                if (x.tc != TC_INT) return false;
                out[0] = 0u - x.w[0];
                return true;
            }
            if (x.n == 3 && nr == 1) return false;
            for (int c = 0; c < nr; ++c)
                if (!put(c, -x.f(c))) return false;
            return true;
        }
        if (n == "compref") {
            if (!cval_of(op.args[1], x) || !cval_of(op.args[2], y) || x.n != 3 || y.tc != TC_INT || rint) return false;
            const int i = (int)(int32_t)y.w[0];
            if (i < 0 || i > 2) return false;
            out[0] = x.w[i];
            return nr == 1;
        }
        if (na < 3 || !cval_of(op.args[1], x) || !cval_of(op.args[2], y)) return false;
        static const std::map<std::string, int> cmp = { { "eq", 0 }, { "neq", 1 }, { "lt", 2 },
                                                        { "gt", 3 }, { "le", 4 }, { "ge", 5 } };
        auto ci = cmp.find(n);
        if (ci != cmp.end()) {
            if (!rint) return false;
            const int K = ci->second;
            bool res;
            if (x.tc == TC_INT && y.tc == TC_INT) {
                const int32_t a = (int32_t)x.w[0], b = (int32_t)y.w[0];
                res = K == 0 ? a == b : K == 1 ? a != b : K == 2 ? a < b : K == 3 ? a > b : K == 4 ? a <= b : a >= b;
            } else if (K <= 1) {
                bool eq = true;
                for (int c = 0; c < std::max(x.n, y.n); ++c) eq = eq && x.f(c) == y.f(c);
                res = K == 0 ? eq : !eq;
            } else {
                const float a = x.f(0), b = y.f(0);
                res = K == 2 ? a < b : K == 3 ? a > b : K == 4 ? a <= b : a >= b;
            }
            out[0] = res ? 1u : 0u;
            return true;
        }
        if (n == "and" || n == "or") {
            if (!rint) return false;
            out[0] = (n == "and" ? (x.truth() && y.truth()) : (x.truth() || y.truth())) ? 1u : 0u;
            return true;
        }
        const int K = n == "add" ? 0 : n == "sub" ? 1 : n == "mul" ? 2 : n == "div" ? 3 : -1;
        if (K < 0) return false;
        if (rint && x.tc == TC_INT && y.tc == TC_INT) {
            const int32_t a = (int32_t)x.w[0], b = (int32_t)y.w[0];
            if (K == 0) out[0] = (uint32_t)a + (uint32_t)b;
            else if (K == 1) out[0] = (uint32_t)a - (uint32_t)b;
            else if (K == 2) out[0] = (uint32_t)a * (uint32_t)b;
            else out[0] = (b == 0 || (a == INT32_MIN && b == -1)) ? 0u : (uint32_t)(a / b);
            return true;
        }
        if ((x.n == 3 || y.n == 3) && nr == 1) return false;
        for (int c = 0; c < nr; ++c) {
            const float a = x.f(c), b = y.f(c);
            float v;
            if (K == 0) v = a + b;
            else if (K == 1) v = a - b;
            else if (K == 2) v = a * b;
            else v = b == 0.0f ? 0.0f : a / b;
            if (!put(c, v)) return false;
        }
        return true;
    }
    void written_in(int b, int e, std::set<int>& w) const {
        for (int k = b; k < e; ++k)
            for (size_t i = 0; i < lops[k].args.size(); ++i)
                if (writes_arg(lops[k], (int)i)) w.insert(lops[k].args[i]);
    }
    int folded_ops = 0;
    // After a return (conditional or not) some points skip the rest of the
    // layer, and after an exit the rest of the group; the output stores still
    // run for exited points. Values known only on the points that went on
    // are dropped at the layer's end (return) or not substituted into the
    // output stores (exit).
    bool fold_ret_div = false, fold_exit_div = false;
    std::set<int> fold_unsafe_ret, fold_unsafe_exit;
    static bool output_stage(const LOp& op) {
        return op.name == "__store_output" || op.name == "__bsdf_eval" || op.name == "__bsdf_sample"
            || op.name == "__store_heap";
    }
    bool range_has(int b, int e, const char* name) const {
        for (int q = b; q < e; ++q)
            if (lops[(size_t)q].name == name) return true;
        return false;
    }
    void fold_written(const LOp& op) {
        for (size_t i = 0; i < op.args.size(); ++i) {
            if (!writes_arg(op, (int)i)) continue;
            if (fold_ret_div) fold_unsafe_ret.insert(op.args[i]);
            if (fold_exit_div) fold_unsafe_exit.insert(op.args[i]);
        }
    }
    void fold_op(LOp& op, std::map<int, int>& K, const std::set<int>& blocked) {
        static const std::set<std::string> control = { "if", "for", "while", "dowhile", "break", "continue",
                                                       "return", "exit", "nop", "useparam", "functioncall",
                                                       "functioncall_nr", "__fret", "__layer_end",
                                                       "__stores_end" };
        if (control.count(op.name) || op.args.empty()) return;
        if (op.param_init) {  // a parameter's uniform value
            if (blocked.count(op.param_gsym)) K.erase(op.param_gsym);
            else K[op.param_gsym] = op.args[1];
            return;
        }
        fold_written(op);
        const bool outs = output_stage(op);
        for (size_t i = 0; i < op.args.size(); ++i) {
            if (writes_arg(op, (int)i) || partial_write(op)) continue;
            if (outs && fold_unsafe_exit.count(op.args[i])) continue;
            auto it = K.find(op.args[i]);
            if (it != K.end()) op.args[i] = it->second;
        }
        std::vector<uint32_t> w;
        if (fold_eval(op, w)) {
            const int r = op.args[0];
            const int c = const_words(syms[r].type, w);
            if (op.name != "assign" || op.args[1] != c) ++folded_ops;
            op.name = "assign";
            op.args = { r, c };
            op.argrw = "wr";
            if (blocked.count(r)) K.erase(r);
            else K[r] = c;
            return;
        }
        for (size_t i = 0; i < op.args.size(); ++i)
            if (writes_arg(op, (int)i)) K.erase(op.args[i]);
    }
    void fold_range(int b, int e, std::map<int, int>& K, const std::set<int>& blocked) {
        for (int k = b; k < e;) {
            LOp& op = lops[k];
            if (op.name == "return") fold_ret_div = true;
            if (op.name == "exit") fold_exit_div = true;
            if (op.name == "__layer_end") {
                for (int s2 : fold_unsafe_ret) K.erase(s2);
                fold_unsafe_ret.clear();
                fold_ret_div = false;
            }
            if (op.name == "functioncall" || op.name == "functioncall_nr") {
                // a body that a return leaves early: what it writes is known
                // only on the points that went on
                const int jend = op.jumps.empty() ? k + 1 : op.jumps[0];
                if (range_has(k + 1, jend, "__fret")) {
                    std::map<int, int> K1 = K;
                    fold_range(k + 1, jend, K1, blocked);
                    std::set<int> w;
                    written_in(k + 1, jend, w);
                    for (int s2 : w) K.erase(s2);
                    k = jend;
                    continue;
                }
                ++k;
                continue;
            }
            if (op.name == "if" && op.jumps.size() >= 2) {
                const int je = op.jumps[0], jend = op.jumps[1];
                // a known condition: the branch not taken never runs; the
                // taken one continues inline as straight-line code
                CVal cv;
                int cs = op.args.empty() ? -1 : op.args[0];
                if (cs >= 0 && K.count(cs)) cs = K[cs];
                if (cs >= 0 && cval_of(cs, cv)) {
                    const bool taken = cv.truth();
                    for (int q = taken ? je : k + 1; q < (taken ? jend : je); ++q) {
                        lops[q].name = "nop";
                        lops[q].args.clear();
                        lops[q].jumps.clear();
                        lops[q].param_init = false;
                    }
                    op.name = "nop";
                    op.args.clear();
                    op.jumps.clear();
                    ++folded_ops;
                    ++k;
                    continue;
                }
                std::map<int, int> K1 = K, K2 = K;
                fold_range(k + 1, je, K1, blocked);
                fold_range(je, jend, K2, blocked);
                std::set<int> w;
                written_in(k + 1, jend, w);
                for (int s : w) K.erase(s);
                k = jend;
                continue;
            }
            if ((op.name == "for" || op.name == "while" || op.name == "dowhile") && op.jumps.size() >= 4) {
                const int jend = op.jumps[3];
                std::set<int> w;
                written_in(k + 1, jend, w);
                for (int s : w) K.erase(s);
                std::set<int> bl = blocked;
                bl.insert(w.begin(), w.end());
                std::map<int, int> K1 = K;
                fold_range(k + 1, jend, K1, bl);
                k = jend;
                continue;
            }
            fold_op(op, K, blocked);
            ++k;
        }
    }
    void fold_constants() {
        std::map<int, int> K;
        fold_range(0, (int)lops.size(), K, std::set<int>());
    }

    // ---- dead-op elimination ----------------------------------------------------
    static bool has_effect(const LOp& op) {
        static const std::set<std::string> effects = {
            "if", "for", "while", "dowhile", "break", "continue", "return", "exit", "__layer_end", "__fret",
            "__stores_end", "__store_heap",
            "__store_output", "__bsdf_eval", "__bsdf_sample", "printf", "warning", "error", "fprintf",
            "functioncall", "functioncall_nr", "useparam", "setmessage", "getmessage" };
        return effects.count(op.name) != 0;
    }
    // ops that update part of their result keep its other components: the
    // result is read as well as written
    static bool partial_write(const LOp& op) {
        return op.name == "compassign" || op.name == "aassign" || op.name == "mxcompassign";
    }
    int eliminate_dead_ops() {
        std::vector<char> needed(syms.size(), 0), live(lops.size(), 0);
        auto take = [&](int k) {
            live[k] = 1;
            const LOp& op = lops[k];
            for (size_t i = 0; i < op.args.size(); ++i)
                if (!writes_arg(op, (int)i) || partial_write(op)) needed[op.args[i]] = 1;
        };
        for (int k = 0; k < (int)lops.size(); ++k)
            if (has_effect(lops[k])) take(k);
        for (bool changed = true; changed;) {
            changed = false;
            for (int k = (int)lops.size() - 1; k >= 0; --k) {
                if (live[k] || lops[k].name == "nop") continue;
                const LOp& op = lops[k];
                for (size_t i = 0; i < op.args.size(); ++i)
                    if (writes_arg(op, (int)i) && needed[op.args[i]]) {
                        take(k);
                        changed = true;
                        break;
                    }
            }
        }
        int removed = 0;
        for (int k = 0; k < (int)lops.size(); ++k)
            if (!live[k] && lops[k].name != "nop") {
                lops[k].name = "nop";
                lops[k].args.clear();
                lops[k].param_init = false;
                ++removed;
            }
        return removed;
    }

    void mark_derivs(int s) {
        if (syms[s].type.derivable() && !syms[s].is_const) syms[s].derivs = true;
    }

    // ---- storage -------------------------------------------------------------
    uint32_t pool_add(const GSym& s) {
        uint32_t off = (uint32_t)pool.size();
        int n = s.type.ncomp() * s.type.elems();
        if (s.type.base == BT_STRING) {
            for (int i = 0; i < s.type.elems(); ++i) {
                std::string v = i < (int)s.sval.size() ? s.sval[i] : std::string();
                pool.push_back(string_hash(v));
            }
            return off;
        }
        for (int i = 0; i < n; ++i) {
            float v = 0.0f;
            if (!s.cval.empty()) v = s.cval[std::min<size_t>(i, s.cval.size() - 1)];
            if (s.type.base == BT_MATRIX && s.cval.size() == 1) v = (i % 5 == 0) ? s.cval[0] : 0.0f;
            if (s.type.base == BT_TRIPLE && s.cval.size() == 1) v = s.cval[0];
            uint32_t w;
            if (s.type.base == BT_INT || s.type.base == BT_CLOSURE) {
                int iv = (int)v;
                std::memcpy(&w, &iv, 4);
            } else {
                std::memcpy(&w, &v, 4);
            }
            pool.push_back(w);
        }
        return off;
    }

    // Live interval of every heap symbol over the linear op list, widened to
    // cover each loop that references it (a value can flow around the back
    // edge). Symbols whose intervals do not overlap share heap slots.
    // ---- static closures ------------------------------------------------------
    // When no closure value depends on control flow (every closure write is
    // outside ifs and loops, there is no return or exit) this pass knows the
    // tree of each closure value: a closure op is a component node; MUL
    // wraps a subtree; ADD joins two. testrender's walk of such a tree
    // (src/testrender/shading.cpp:1450-1500) visits the components in a
    // fixed order, each with the product of the MUL weights above it, and a
    // zero MUL weight or a zero component weight removes the subtree (the
    // reference returns null closures, src/liboslexec/opclosure.cpp:15-117).
    // So each closure op becomes a node at a fixed heap slot, MUL weights are
    // kept, ADD and closure assignment disappear, and each consumer (record
    // store, BSDF eval or sample) receives the walk unrolled as a term table
    // whose weights and presence flags are computed by ordinary ops in the
    // walk's order. Results are those of the tree walk.
    struct ClTerm {
        int node;                // the component's node block (gsym)
        std::vector<int> chain;  // MUL weight gsyms, outermost first
    };
    bool closure_consumer(const LOp& op) const {
        if (op.name == "__bsdf_eval" || op.name == "__bsdf_sample") return true;
        return op.name == "__store_output" && !op.args.empty() && is_closure(op.args[0]);
    }
    bool closure_writer(const LOp& op) const {
        if (op.args.empty() || !is_closure(op.args[0])) return false;
        return op.name == "closure" || op.name == "add" || op.name == "mul" || op.name == "assign";
    }
    // a weight known to be zero (every component 0) or known to be nonzero
    int const_zero(int gs) const {
        CVal v;
        if (!cval_of(gs, v)) return -1;
        for (int c = 0; c < v.n; ++c) {
            const float x = v.f(c);
            if (x != 0.0f || x != x) return 0;
        }
        return 1;
    }
    int none_sym = -1;
    int new_sym(const std::string& name, BaseType b, int arraylen = 0, VecSem vs = VS_NONE) {
        GSym t;
        t.name = name;
        t.type.base = b;
        t.type.arraylen = arraylen;
        t.type.vecsem = vs;
        t.kind = SK_LOCAL;
        return add_sym(t);
    }
    bool static_closures() {
        if (!ss.opts.opt_static_closures) return false;
        const int n = (int)lops.size();
        std::vector<int> depth(n + 1, 0);
        bool any = false;
        for (int k = 0; k < n; ++k) {
            const LOp& op = lops[k];
            int end = -1;
            if (op.name == "if" && op.jumps.size() >= 2) end = op.jumps[1];
            else if ((op.name == "for" || op.name == "while" || op.name == "dowhile") && op.jumps.size() >= 4)
                end = op.jumps[3];
            for (int j = k + 1; j < std::min(end, n); ++j) depth[j]++;
            for (int a : op.args)
                if (is_closure(a)) {
                    any = true;
                    if (syms[a].type.is_array()) return false;
                }
        }
        if (!any) return false;
        // eligibility, and a dry run of the term lists
        std::map<int, std::vector<ClTerm>> val;
        int adds = 0;
        for (int k = 0; k < n; ++k) {
            const LOp& op = lops[k];
            if (op.name == "return" || op.name == "exit" || op.name == "__fret") return false;
            bool refs = false;
            for (int a : op.args) refs = refs || is_closure(a);
            if (!refs || op.name == "useparam") continue;
            if (closure_consumer(op)) {
                if (depth[k]) return false;
                // a BSDF consumer keeps one lobe position per term
                const size_t cap = op.name == "__store_output" ? kMaxStaticTerms : kBsdfMaxLobes;
                if (val[op.args[0]].size() > cap) return false;
                continue;
            }
            if (!closure_writer(op) || depth[k]) return false;
            const int r = op.args[0];
            if (op.name == "closure") {
                // closures taking closures (layer) keep the run-time tree
                for (size_t i = 1; i < op.args.size(); ++i)
                    if (is_closure(op.args[i])) return false;
                val[r] = { ClTerm{ -1, {} } };
            } else if (op.name == "assign") {
                val[r] = op.args.size() > 1 && is_closure(op.args[1]) ? val[op.args[1]] : std::vector<ClTerm>{};
            } else if (op.name == "add") {
                if (op.args.size() < 3 || !is_closure(op.args[1]) || !is_closure(op.args[2])) return false;
                std::vector<ClTerm> t = val[op.args[1]];
                for (const ClTerm& x : val[op.args[2]]) t.push_back(x);
                val[r] = t;
                ++adds;
            } else {  // mul
                if (op.args.size() < 3) return false;
                const int c = is_closure(op.args[1]) ? op.args[1] : op.args[2];
                val[r] = val[c];
            }
            if (val[r].size() > 64) return false;
        }
        // the reference walk keeps at most this many pending branches
        if (adds > kClosureWalkStack) return false;

        // the rewrite
        GSym nn;
        nn.name = "$noarg";
        nn.type.base = BT_INT;
        nn.kind = SK_CONST;
        nn.is_const = true;
        nn.cval = { 0.0f };
        none_sym = add_sym(nn);
        val.clear();
        std::vector<LOp> out;
        std::vector<int> newpos(n + 1, 0);
        for (int k = 0; k < n; ++k) {
            newpos[k] = (int)out.size();
            const LOp& op = lops[k];
            if (closure_writer(op)) {
                const int r = op.args[0];
                if (op.name == "closure") {
                    const int b = new_sym("$clnode", BT_FLOAT,
                                          closure_param_words(op) > kRecordParams ? kNodeFloats : kRecordFloats);
                    LOp nd = op;
                    nd.name = "__cl_node";
                    nd.args[0] = b;
                    nd.argrw.clear();
                    out.push_back(nd);
                    val[r] = { ClTerm{ b, {} } };
                } else if (op.name == "assign") {
                    val[r] = op.args.size() > 1 && is_closure(op.args[1]) ? val[op.args[1]] : std::vector<ClTerm>{};
                } else if (op.name == "add") {
                    std::vector<ClTerm> t = val[op.args[1]];
                    for (const ClTerm& x : val[op.args[2]]) t.push_back(x);
                    val[r] = t;
                } else {  // mul: keep the weight as it is now
                    const bool cfirst = is_closure(op.args[1]);
                    const int c = cfirst ? op.args[1] : op.args[2];
                    int w = cfirst ? op.args[2] : op.args[1];
                    std::vector<ClTerm> t;
                    const int z = const_zero(w);
                    if (z != 1) {  // a zero weight leaves the null closure
                        if (!syms[w].is_const) {
                            const int cap = new_sym("$clw", syms[w].type.base, 0, syms[w].type.vecsem);
                            LOp as;
                            as.name = "assign";
                            as.layer = op.layer;
                            as.args = { cap, w };
                            out.push_back(as);
                            w = cap;
                        }
                        for (const ClTerm& x : val[c]) {
                            ClTerm y{ x.node, { w } };
                            for (int m : x.chain) y.chain.push_back(m);
                            t.push_back(y);
                        }
                    }
                    val[r] = t;
                }
                continue;
            }
            if (closure_consumer(op)) {
                // per term: its weight product and presence, then the consumer
                LOp cons = op;
                cons.argrw.clear();
                cons.name = op.name == "__store_output" ? "__cl_store"
                          : op.name == "__bsdf_eval"    ? "__cl_bsdf_eval"
                                                        : "__cl_bsdf_sample";
                cons.args.erase(cons.args.begin());
                cons.imm[3] = op.imm[3];
                for (const ClTerm& t : val[op.args[0]]) {
                    int cw = none_sym, pres = none_sym;
                    if (!t.chain.empty()) {
                        const int acc = new_sym("$clacc", BT_TRIPLE, 0, VS_COLOR);
                        LOp a0;
                        a0.name = "assign";
                        a0.args = { acc, t.chain[0] };
                        out.push_back(a0);
                        for (size_t j = 1; j < t.chain.size(); ++j) {
                            LOp m;
                            m.name = "mul";
                            m.args = { acc, acc, t.chain[j] };
                            out.push_back(m);
                        }
                        cw = new_sym("$clcw", BT_TRIPLE, 0, VS_COLOR);
                        LOp mn;
                        mn.name = "__cl_mulnode";
                        mn.args = { cw, acc, t.node };
                        out.push_back(mn);
                        for (int m : t.chain) {
                            if (const_zero(m) == 0) continue;  // a constant nonzero weight
                            const int zero = syms[m].type.base == BT_TRIPLE
                                               ? const_triple_sym({ 0.0f, 0.0f, 0.0f })
                                               : const_float(0.0f);
                            const int ne = new_sym("$clnz", BT_INT);
                            LOp q;
                            q.name = "neq";
                            q.args = { ne, m, zero };
                            out.push_back(q);
                            if (pres == none_sym) {
                                pres = ne;
                            } else {
                                LOp an;
                                an.name = "and";
                                an.args = { pres, pres, ne };
                                out.push_back(an);
                            }
                        }
                    }
                    cons.args.push_back(t.node);
                    cons.args.push_back(cw);
                    cons.args.push_back(pres);
                }
                out.push_back(cons);
                continue;
            }
            out.push_back(op);
        }
        newpos[n] = (int)out.size();
        for (LOp& op : out)
            for (int& j : op.jumps) j = newpos[std::min(std::max(j, 0), n)];
        lops = std::move(out);
        return true;
    }
    // a color constant created before storage assignment (no pool slot yet)
    int const_triple_sym(const std::array<float, 3>& v) {
        GSym d;
        d.name = "$triple";
        d.type.base = BT_TRIPLE;
        d.type.vecsem = VS_COLOR;
        d.kind = SK_CONST;
        d.is_const = true;
        d.cval = { v[0], v[1], v[2] };
        return add_sym(d);
    }

    void assign_storage() {
        for (const LOp& op : lops)
            for (int a : op.args) syms[a].referenced = true;
        const int n = (int)lops.size();
        std::vector<int> first(syms.size(), n), last(syms.size(), -1);
        for (int k = 0; k < n; ++k)
            for (int a : lops[k].args) {
                first[a] = std::min(first[a], k);
                last[a] = std::max(last[a], k);
            }
        // loops as [begin, end] op ranges
        std::vector<std::pair<int, int>> loops;
        for (int k = 0; k < n; ++k) {
            const LOp& op = lops[k];
            if ((op.name == "for" || op.name == "while" || op.name == "dowhile") && op.jumps.size() >= 4)
                loops.push_back({ k, op.jumps[3] });
        }
        for (size_t si = 0; si < syms.size(); ++si) {
            if (last[si] < 0) continue;
            bool changed = true;
            while (changed) {
                changed = false;
                for (auto& L : loops) {
                    bool touches = !(last[si] < L.first || first[si] > L.second);
                    if (touches && (first[si] > L.first || last[si] < L.second)) {
                        first[si] = std::min(first[si], L.first);
                        last[si] = std::max(last[si], L.second);
                        changed = true;
                    }
                }
            }
        }
        // globals are loaded and message states cleared before op 0; keep
        // them live from the start
        for (auto& kv : globals)
            if (syms[kv.second].referenced) first[kv.second] = -1;
        for (auto& kv : msg_state)
            if (syms[kv.second].referenced) first[kv.second] = -1;
        std::vector<int> order;
        for (size_t si = 0; si < syms.size(); ++si) {
            GSym& s = syms[si];
            if (!s.referenced) continue;
            if (s.is_const) {
                if (s.slot < 0) s.slot = (int)pool_add(s);  // folded values already sit in the pool
                continue;
            }
            order.push_back((int)si);
        }
        std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return first[a] < first[b]; });
        // first-fit reuse of freed slot ranges with the same size
        std::multimap<int, uint32_t> free_by_size;          // size -> slot
        std::multimap<int, std::pair<int, int>> active;     // last use -> (sym, size)
        for (int si : order) {
            GSym& s = syms[si];
            int sz = s.type.ncomp() * s.type.elems() * (s.derivs ? 3 : 1);
            if (s.type.base == BT_VOID) sz = 0;
            while (!active.empty() && active.begin()->first < first[si]) {
                auto it = active.begin();
                free_by_size.insert({ it->second.second, (uint32_t)syms[it->second.first].slot });
                active.erase(it);
            }
            auto f = free_by_size.find(sz);
            if (f != free_by_size.end()) {
                s.slot = (int)f->second;
                free_by_size.erase(f);
            } else {
                s.slot = (int)heap_top;
                heap_top += (uint32_t)sz;
            }
            active.insert({ last[si], { si, sz } });
        }
        // closure node pool: one node per closure-creating op when none sits
        // inside a loop (each op makes at most one node, so the pool cannot
        // overflow), else the configured capacity
        int nclosure_ops = 0;
        bool closure_in_loop = false;
        for (int k = 0; k < n; ++k) {
            const LOp& op = lops[k];
            bool creates = op.name == "closure"
                        || ((op.name == "mul" || op.name == "add") && !op.args.empty()
                            && syms[op.args[0]].type.base == BT_CLOSURE);
            if (!creates) continue;
            ++nclosure_ops;
            for (auto& L : loops)
                if (k > L.first && k < L.second) closure_in_loop = true;
        }
        closure_nodes = closure_in_loop ? ss.opts.max_closure_components : nclosure_ops;
        if (closure_nodes < 1) closure_nodes = 1;
    }
    int closure_nodes = 0;

    uint32_t A(int gs) {
        const GSym& s = syms[gs];
        return arg_make((uint32_t)s.slot, s.is_const, s.derivs, s.type.tclass());
    }

    // ---- emission ------------------------------------------------------------
    int emit(uint16_t code, std::initializer_list<uint32_t> a, const std::string& name) {
        Op op;
        std::memset(&op, 0, sizeof(op));
        op.code = code;
        int i = 0;
        for (uint32_t v : a) {
            if (i < 7) op.a[i++] = v;
        }
        op.nargs = (uint8_t)i;
        ops.push_back(op);
        op_names.push_back(name);
        return (int)ops.size() - 1;
    }

    bool emit_range(int b, int e, int depth, int loopl, int funcl = 0) {
        for (int k = b; k < e;) {
            const LOp& op = lops[k];
            if (op.name == "functioncall" || op.name == "functioncall_nr") {
                // a user function's inlined body (oslc, codegen.cpp:1890-1905):
                // masked like a block when a return inside ends it early
                const int jend = op.jumps.empty() ? k + 1 : op.jumps[0];
                if (jend <= k || jend > e) return fail("functioncall with a bad end");
                bool early = false;
                for (int q = k + 1; q < jend; ++q) early = early || (lops[q].name == "__fret" && lops[q].imm[0] == k);
                if (!early) {
                    if (!emit_range(k + 1, jend, depth, loopl, funcl)) return false;
                    k = jend;
                    continue;
                }
                if ((uint32_t)depth + 1 > max_depth) max_depth = depth + 1;
                if (depth >= 31) return fail("control flow nested too deeply");
                const uint32_t tag = (uint32_t)depth + 1;
                const int beg = emit(OP_FUNC_BEGIN, { 0u, (uint32_t)depth, 0u, tag }, "functioncall");
                const size_t first_ret = fret_ops.size();
                if (!emit_range(k + 1, jend, depth + 1, loopl, (int)tag)) return false;
                const int endop = emit(OP_FUNC_END, { 0u, (uint32_t)depth, 0u, tag }, "functioncall");
                ops[beg].a[2] = (uint32_t)endop;
                for (size_t q = first_ret; q < fret_ops.size(); ++q)
                    if (ops[fret_ops[q]].a[3] == tag) ops[fret_ops[q]].a[2] = (uint32_t)endop;
                k = jend;
                continue;
            }
            if (op.name == "if") {
                if (op.jumps.size() < 2) return fail("if without jump targets");
                int je = op.jumps[0], jend = op.jumps[1];
                if ((uint32_t)depth + 1 > max_depth) max_depth = depth + 1;
                if (depth >= 31) return fail("control flow nested too deeply");
                int ifop = emit(OP_IF, { A(op.args[0]), (uint32_t)depth, 0u, (uint32_t)loopl }, "if");
                if (!emit_range(k + 1, je, depth + 1, loopl, funcl)) return false;
                int elop = emit(OP_ELSE, { 0u, (uint32_t)depth, 0u, (uint32_t)loopl }, "if");
                ops[ifop].a[2] = (uint32_t)elop;
                if (!emit_range(je, jend, depth + 1, loopl, funcl)) return false;
                int enop = emit(OP_ENDIF, { 0u, (uint32_t)depth, 0u, (uint32_t)loopl }, "if");
                ops[elop].a[2] = (uint32_t)enop;
                k = jend;
                continue;
            }
            if (op.name == "for" || op.name == "while" || op.name == "dowhile") {
                if (op.jumps.size() < 4) return fail(op.name + " without jump targets");
                int jc = op.jumps[0], jb = op.jumps[1], js = op.jumps[2], jend = op.jumps[3];
                if ((uint32_t)depth + 1 > max_depth) max_depth = depth + 1;
                if (depth >= 31) return fail("control flow nested too deeply");
                uint32_t ll = (uint32_t)depth + 1;  // loop level tag = its depth + 1
                emit(OP_LOOP_BEGIN, { 0u, (uint32_t)depth, 0u, ll }, op.name);
                if (!emit_range(k + 1, jc, depth + 1, (int)ll, funcl)) return false;
                int jmp_body = -1;
                if (op.name == "dowhile") jmp_body = emit(OP_JUMP, { 0u, 0u, 0u, 0u }, op.name);
                int cond_start = (int)ops.size();
                if (!emit_range(jc, jb, depth + 1, (int)ll, funcl)) return false;
                int test = emit(OP_LOOP_TEST, { A(op.args[0]), (uint32_t)depth, 0u, ll }, op.name);
                if (jmp_body >= 0) ops[jmp_body].a[2] = (uint32_t)ops.size();
                if (!emit_range(jb, js, depth + 1, (int)ll, funcl)) return false;
                emit(OP_LOOP_STEP, { 0u, (uint32_t)depth, 0u, ll }, op.name);
                if (!emit_range(js, jend, depth + 1, (int)ll, funcl)) return false;
                emit(OP_JUMP, { 0u, 0u, (uint32_t)cond_start, 0u }, op.name);
                int endop = emit(OP_LOOP_END, { 0u, (uint32_t)depth, 0u, ll }, op.name);
                ops[test].a[2] = (uint32_t)endop;
                k = jend;
                continue;
            }
            if (op.name == "__fret") {  // return from the enclosing user function
                if (!funcl) return fail("internal: function return outside a function body");
                fret_ops.push_back(emit(OP_FUNC_RETURN, { 0u, 0u, 0u, (uint32_t)funcl }, "return"));
                ++k;
                continue;
            }
            if (!lower_op(op, depth, loopl)) return false;
            ++k;
        }
        return true;
    }

    bool lower_all() {
        // global loads first
        for (auto& kv : globals) {
            const GSym& s = syms[kv.second];
            if (!s.referenced) continue;
            if (s.global_id < 0) {
                if (s.type.base == BT_CLOSURE) {
                    // Ci and other closure globals start as the null closure
                    int z = const_int(0);
                    syms[z].slot = (int)pool_add(syms[z]);
                    emit(OP_ASSIGN, { A(kv.second), A(z), 1u }, "global");
                    continue;
                }
                return fail("shader global '" + s.name + "' is not supported");
            }
            emit(OP_LOAD_GLOBAL, { A(kv.second), (uint32_t)s.global_id }, "global");
        }
        // every message starts unset
        for (auto& kv : msg_state) {
            if (!syms[kv.second].referenced) continue;
            int z = const_int(0);
            syms[z].slot = (int)pool_add(syms[z]);
            emit(OP_ASSIGN, { A(kv.second), A(z), 1u, 1u, 1u }, "message");
        }
        // the body of each layer is a structured range of lops
        if (!emit_range(0, (int)lops.size(), 0, 0)) return false;
        return check_destinations();
    }

    // Every op that writes its first operand must write a heap slot: a
    // constant there would mean a write into the constant pool's offsets.
    bool check_destinations() {
        for (size_t k = 0; k < ops.size(); ++k) {
            const Op& o = ops[k];
            switch (o.code) {
            case OP_NOP: case OP_IF: case OP_ELSE: case OP_ENDIF: case OP_LOOP_BEGIN: case OP_LOOP_TEST:
            case OP_LOOP_STEP: case OP_LOOP_END: case OP_JUMP: case OP_BREAK: case OP_CONTINUE: case OP_RETURN:
            case OP_EXIT: case OP_LAYER_END: case OP_STORE_OUTPUT: case OP_STORE_CLOSURE: case OP_BSDF_EVAL:
            case OP_BSDF_SAMPLE: case OP_CL_STORE: case OP_CL_BSDF_EVAL: case OP_CL_BSDF_SAMPLE:
            case OP_FUNC_BEGIN: case OP_FUNC_RETURN: case OP_FUNC_END: case OP_STORES_END: case OP_STORE_HEAP:
                continue;
            default:
                break;
            }
            bool bad = (o.a[0] & kArgConst) != 0;
            if (o.code == OP_SETMESSAGE) bad = bad || (o.a[1] & kArgConst) != 0;
            if (o.code == OP_GETMESSAGE) bad = bad || (o.a[3] & kArgConst) != 0;
            if (bad) return fail("internal: op '" + op_names[k] + "' would write a constant");
        }
        return true;
    }

    int tc(int gs) const { return (int)syms[gs].type.tclass(); }
    bool is_int(int gs) const { return syms[gs].type.base == BT_INT; }
    bool is_closure(int gs) const { return syms[gs].type.base == BT_CLOSURE; }
    bool is_matrix(int gs) const { return syms[gs].type.base == BT_MATRIX; }
    bool is_triple(int gs) const { return syms[gs].type.base == BT_TRIPLE; }
    bool is_string(int gs) const { return syms[gs].type.base == BT_STRING; }
    // Parameter words the device's closure_fill writes for closure op `op`
    // (an upper bound): each operand's components, at most 16, at most
    // kClosureParamFloats in all.
    // The BSDF code reads a lobe's fixed parameter words where they must be
    // (testrender's parameter structs, shading.h:66-211, and BSDL's lobe
    // Data): a closure op with fewer is refused rather than read past.
    bool closure_params_complete(const std::string& cname, const LOp& op) {
        static const std::map<std::string, int> fixed = {
            { "diffuse", 3 }, { "oren_nayar", 4 }, { "microfacet", 11 }, { "oren_nayar_diffuse_bsdf", 7 },
            { "sheen_bsdf", 7 }, { "dielectric_bsdf", 16 } };
        auto it = fixed.find(cname);
        if (it == fixed.end() || closure_param_words(op) >= it->second) return true;
        return fail("closure '" + cname + "' needs " + std::to_string(it->second) + " parameter words, has " +
                    std::to_string(closure_param_words(op)));
    }
    int closure_param_words(const LOp& op) const {
        const size_t na = op.args.size();
        size_t ni = 1;
        if (na > 1 && !is_string(op.args[1])) ni = 2;
        int w = 0;
        for (size_t i = ni + 1; i < na && i < ni + 12; ++i) {
            const TypeSpec& t = syms[op.args[i]].type;
            w += std::min(16, std::max(1, t.ncomp() * t.elems()));
        }
        return std::min(w, kClosureParamFloats);
    }

    std::string const_string(int gs) const {
        const GSym& s = syms[gs];
        if (s.is_const && !s.sval.empty()) return s.sval[0];
        return std::string();
    }

    // Rec709 colour system as ColorSystem::set_colorspace derives it
    // (src/liboslexec/opcolor.cpp:140-190): XYZ->RGB from the primaries and
    // the D65 white point, and the luminance weights = the middle column of
    // its inverse (cofactors over the determinant).
    struct ColorSys {
        float xyz2rgb[3][3];  // row-vector convention: rgb = XYZ * M
        float rgb2xyz[3][3];  // its inverse, cofactors over the determinant (Imath Matrix33::inverse)
        std::array<float, 3> lum;
    };
    // The colour systems ColorSystem knows by name (src/liboslexec/opcolor.cpp:
    // 31-85): red, green, blue and white chromaticities (published standard
    // primaries; IlluminantC/D65/E/ACES white points).
    struct Chroma {
        const char* name;
        float xr, yr, xg, yg, xb, yb, xw, yw;
    };
    static const Chroma* chroma_of(const std::string& name) {
        static const Chroma k[] = {
            { "Rec709", 0.64f, 0.33f, 0.30f, 0.60f, 0.15f, 0.06f, 0.3127f, 0.3291f },
            { "sRGB", 0.64f, 0.33f, 0.30f, 0.60f, 0.15f, 0.06f, 0.3127f, 0.3291f },
            { "NTSC", 0.67f, 0.33f, 0.21f, 0.71f, 0.14f, 0.08f, 0.3101f, 0.3162f },
            { "EBU", 0.64f, 0.33f, 0.29f, 0.60f, 0.15f, 0.06f, 0.3127f, 0.3291f },
            { "PAL", 0.64f, 0.33f, 0.29f, 0.60f, 0.15f, 0.06f, 0.3127f, 0.3291f },
            { "SECAM", 0.64f, 0.33f, 0.29f, 0.60f, 0.15f, 0.06f, 0.3127f, 0.3291f },
            { "SMPTE", 0.630f, 0.340f, 0.310f, 0.595f, 0.155f, 0.070f, 0.3127f, 0.3291f },
            { "HDTV", 0.670f, 0.330f, 0.210f, 0.710f, 0.150f, 0.060f, 0.3127f, 0.3291f },
            { "CIE", 0.7355f, 0.2645f, 0.2658f, 0.7243f, 0.1669f, 0.0085f, 0.33333333f, 0.33333333f },
            { "AdobeRGB", 0.64f, 0.33f, 0.21f, 0.71f, 0.15f, 0.06f, 0.3127f, 0.3291f },
            { "XYZ", 1.0f, 0.0f, 0.0f, 1.0f, 0.0f, 0.0f, 0.33333333f, 0.33333333f },
            { "ACES2065-1", 0.7347f, 0.2653f, 0.0f, 1.0f, 0.0001f, -0.077f, 0.32168f, 0.33767f },
            { "ACEScg", 0.713f, 0.293f, 0.165f, 0.83f, 0.128f, 0.044f, 0.32168f, 0.33767f },
        };
        for (const Chroma& c : k)
            if (name == c.name) return &c;
        return nullptr;
    }
    static ColorSys make_color_system(const Chroma& ch) {
        ColorSys c;
        const float xr = ch.xr, yr = ch.yr, xg = ch.xg, yg = ch.yg, xb = ch.xb, yb = ch.yb, xw = ch.xw, yw = ch.yw;
        const float R[3] = { xr, yr, 1.0f - (xr + yr) }, G[3] = { xg, yg, 1.0f - (xg + yg) },
                    B[3] = { xb, yb, 1.0f - (xb + yb) }, W[3] = { xw, yw, 1.0f - (xw + yw) };
        float r[3] = { G[1] * B[2] - B[1] * G[2], B[0] * G[2] - G[0] * B[2], G[0] * B[1] - B[0] * G[1] };
        float g[3] = { B[1] * R[2] - R[1] * B[2], R[0] * B[2] - B[0] * R[2], B[0] * R[1] - R[0] * B[1] };
        float b[3] = { R[1] * G[2] - G[1] * R[2], G[0] * R[2] - R[0] * G[2], R[0] * G[1] - G[0] * R[1] };
        float w[3] = { r[0] * W[0] + r[1] * W[1] + r[2] * W[2], g[0] * W[0] + g[1] * W[1] + g[2] * W[2],
                       b[0] * W[0] + b[1] * W[1] + b[2] * W[2] };
        if (W[1] != 0.0f) {
            const float ws = 1.0f / W[1];
            for (float& x : w) x *= ws;
        }
        for (int i = 0; i < 3; ++i) { r[i] /= w[0]; g[i] /= w[1]; b[i] /= w[2]; }
        const float M[3][3] = { { r[0], g[0], b[0] }, { r[1], g[1], b[1] }, { r[2], g[2], b[2] } };
        std::memcpy(c.xyz2rgb, M, sizeof(M));
        float C[3][3];  // adjugate
        C[0][0] = M[1][1] * M[2][2] - M[2][1] * M[1][2];
        C[0][1] = M[2][1] * M[0][2] - M[0][1] * M[2][2];
        C[0][2] = M[0][1] * M[1][2] - M[1][1] * M[0][2];
        C[1][0] = M[2][0] * M[1][2] - M[1][0] * M[2][2];
        C[1][1] = M[0][0] * M[2][2] - M[2][0] * M[0][2];
        C[1][2] = M[1][0] * M[0][2] - M[0][0] * M[1][2];
        C[2][0] = M[1][0] * M[2][1] - M[2][0] * M[1][1];
        C[2][1] = M[2][0] * M[0][1] - M[0][0] * M[2][1];
        C[2][2] = M[0][0] * M[1][1] - M[1][0] * M[0][1];
        const float det = M[0][0] * C[0][0] + M[0][1] * C[1][0] + M[0][2] * C[2][0];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) c.rgb2xyz[i][j] = C[i][j] / det;
        c.lum = { C[0][1] / det, C[1][1] / det, C[2][1] / det };
        const float lum2 = 1.0f - c.lum[0] - c.lum[1];
        if (std::fabs(lum2 - c.lum[2]) < 0.001f) c.lum[2] = lum2;
        return c;
    }
    // the system's colour space (attribute "colorspace"), derived as
    // ColorSystem::set_colorspace does (src/liboslexec/opcolor.cpp:140-190)
    const ColorSys& csys() const {
        static std::mutex mu;
        static std::map<std::string, ColorSys> cache;
        std::lock_guard<std::mutex> lock(mu);
        auto it = cache.find(ss.opts.colorspace);
        if (it != cache.end()) return it->second;
        const Chroma* ch = chroma_of(ss.opts.colorspace);
        return cache[ss.opts.colorspace] = make_color_system(ch ? *ch : *chroma_of("Rec709"));
    }
    std::array<float, 3> luminance_scale() const { return csys().lum; }

    // Blackbody table (src/liboslexec/opcolor.cpp:191-205,
    // opcolor_impl.h:131-260): Planck spectra at temperatures
    // T_i = 2 i^1.5 + 800 up to 12000 K, integrated against the CIE 1931
    // matching functions, converted to RGB, clamped at zero and stored to
    // the power 1/5. Followed by the XYZ->RGB matrix and the CIE table for
    // temperatures past the table. expm1, cbrt and pow are evaluated in double precision
    // (the reference uses OIIO's fast approximations).
    const std::vector<float>& blackbody_pool() const {
        static std::mutex mu;
        static std::map<std::string, std::vector<float>> cache;
        std::lock_guard<std::mutex> lock(mu);
        auto found = cache.find(ss.opts.colorspace);
        if (found != cache.end()) return found->second;
        const ColorSys& cs = csys();
        std::vector<float>& pool = cache[ss.opts.colorspace];
        pool = [&]() {
            std::vector<float> t;
            float lastT = 0.0f;
            for (int i = 0; lastT <= 12000.0f; ++i) {
                const float is = std::sqrt((float)i);
                const float T = is * is * is * 2.0f + 800.0f;
                lastT = T;
                float rgb[3];
                blackbody_spectral_rgb(T, cs, rgb);
                for (int c = 0; c < 3; ++c) t.push_back((float)std::pow((double)rgb[c], (double)(1.0f / 5.0f)));
            }
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) t.push_back(cs.xyz2rgb[i][j]);
            for (int i = 0; i < 81; ++i)
                for (int j = 0; j < 3; ++j) t.push_back(kCIE[i][j]);
            return t;
        }();
        return pool;
    }
    // compute_blackbody_rgb (opcolor_impl.h:557-566)
    static void blackbody_spectral_rgb(float T, const ColorSys& cs, float* rgb) {
        float X = 0.0f, Y = 0.0f, Z = 0.0f;
        const float dlambda = (float)(5.0f * 1e-9);
        for (int i = 0; i < 81; ++i) {
            const float lambda = 380.0f + 5.0f * (float)i;
            const float wlm = lambda * 1e-9f;
            const float wlm2 = wlm * wlm, wlm4 = wlm2 * wlm2, wlm5 = wlm4 * wlm;
            const float inv5 = 1.0f / wlm5;
            const float e = (float)std::expm1((double)(1.4388e-2f / (wlm * T)));
            const float Me = ((3.74183e-16f * inv5) / e) * dlambda;
            X += Me * kCIE[i][0];
            Y += Me * kCIE[i][1];
            Z += Me * kCIE[i][2];
        }
        for (int c = 0; c < 3; ++c) {
            float v = X * cs.xyz2rgb[0][c] + Y * cs.xyz2rgb[1][c] + Z * cs.xyz2rgb[2][c];
            rgb[c] = v < 0.0f ? 0.0f : v;
        }
    }
    int const_floats(const std::vector<float>& v) {
        GSym d;
        d.name = "$table";
        d.type.base = BT_FLOAT;
        d.type.arraylen = (int)v.size();
        d.kind = SK_CONST;
        d.is_const = true;
        d.cval = v;
        int k = add_sym(d);
        syms[k].slot = (int)pool_add(syms[k]);
        return k;
    }
    int const_triple(const std::array<float, 3>& v) {
        GSym d;
        d.name = "$triple";
        d.type.base = BT_TRIPLE;
        d.type.vecsem = VS_COLOR;
        d.kind = SK_CONST;
        d.is_const = true;
        d.cval = { v[0], v[1], v[2] };
        int k = add_sym(d);
        syms[k].slot = (int)pool_add(syms[k]);
        return k;
    }

    bool lower_noise(const LOp& op) {
        // noise-family ops: (result, [name], S, [T], [Speriod, [Tperiod]], [options...])
        // name mapping follows src/liboslexec/batched_llvm_gen.cpp:6094-6146
        bool periodic = op.name == "pnoise" || op.name == "psnoise";
        size_t ai = 1;
        std::string name;
        if (op.args.size() > 1 && is_string(op.args[1])) {
            name = const_string(op.args[1]);
            if (name.empty() && !syms[op.args[1]].is_const)
                return fail("noise type must be a constant string in this executor");
            ai = 2;
        } else {
            name = op.name;
        }
        int R = op.args[0];
        if (ai >= op.args.size()) return fail("noise op without coordinates");
        int S = op.args[ai++];
        int T = -1, Sp = -1, Tp = -1;
        int dims = is_triple(S) ? 3 : 1;
        if (periodic) {
            if (ai + 1 < op.args.size() && !is_string(op.args[ai + 1])
                && (syms[op.args[ai]].type.base == BT_FLOAT || is_triple(op.args[ai]))
                && (syms[op.args[ai]].type.base == BT_FLOAT)) {
                T = op.args[ai++];
                ++dims;
            }
            if (ai < op.args.size()) Sp = op.args[ai++];
            if ((dims == 2 || dims == 4) && ai < op.args.size()) Tp = op.args[ai++];
        } else if (ai < op.args.size() && syms[op.args[ai]].type.base == BT_FLOAT) {
            T = op.args[ai++];
            ++dims;
        }
        uint32_t kind;
        if (name == "perlin" || name == "snoise" || name == "psnoise") kind = NK_PERLIN;
        else if (name == "uperlin" || name == "noise" || name == "pnoise") kind = NK_UPERLIN;
        else if (name == "cell" || name == "cellnoise") kind = NK_CELL;
        else if (name == "hash" || name == "hashnoise") kind = NK_HASH;
        else if (name == "simplex" && !periodic) kind = NK_SIMPLEX;
        else if (name == "usimplex" && !periodic) kind = NK_USIMPLEX;
        else if (name == "gabor") kind = NK_GABOR;
        else if (name == "null") kind = NK_NULL;
        else if (name == "unull") kind = NK_UNULL;
        else return fail("noise type \"" + name + "\" is unknown");
        bool derivs = syms[R].derivs && (syms[S].derivs || (T >= 0 && syms[T].derivs));
        if (kind == NK_CELL || kind == NK_HASH) derivs = false;
        if (kind == NK_GABOR) {
            // options follow as (name, value) pairs; supported subset lowered
            // into fixed operands: anisotropic, direction, bandwidth, impulses, do_filter
            int aniso = const_int(0), dir = -1, bw = const_float(1.0f), imp = const_float(16.0f),
                filt = const_int(1);
            for (; ai + 1 < op.args.size(); ai += 2) {
                std::string on = const_string(op.args[ai]);
                int v = op.args[ai + 1];
                if (on == "anisotropic") aniso = v;
                else if (on == "direction") dir = v;
                else if (on == "bandwidth") bw = v;
                else if (on == "impulses") imp = v;
                else if (on == "do_filter") filt = v;
            }
            if (dir < 0) {
                GSym d; d.name = "$dir"; d.type.base = BT_TRIPLE; d.type.vecsem = VS_VECTOR;
                d.kind = SK_CONST; d.is_const = true; d.cval = { 1.0f, 0.0f, 0.0f };
                dir = add_sym(d);
                syms[dir].slot = (int)pool_add(syms[dir]);
            }
            for (int x : { aniso, bw, imp, filt })
                if (syms[x].slot < 0) syms[x].slot = (int)pool_add(syms[x]);
            // pack the option operands: a4 = anisotropic(int) a5 = direction a6 = bandwidth
            // impulses and do_filter go in a second op word pair via OP_NOP carrier
            uint32_t kw = noise_word(kind, periodic, dims, is_triple(R), true);
            emit(OP_GABOR, { A(R), A(S), T >= 0 ? A(T) : kNoArg, kw, A(aniso), A(dir), A(bw) }, op.name);
            emit(OP_NOP, { A(imp), A(filt), Sp >= 0 ? A(Sp) : kNoArg, Tp >= 0 ? A(Tp) : kNoArg },
                 "gabor-options");
            return true;
        }
        uint32_t kw = noise_word(kind, periodic, dims, is_triple(R), derivs);
        emit(OP_NOISE, { A(R), A(S), T >= 0 ? A(T) : kNoArg, kw, Sp >= 0 ? A(Sp) : kNoArg,
                         Tp >= 0 ? A(Tp) : kNoArg },
             op.name);
        return true;
    }

    // texture r filename s t ["option", value]... (osl_texture,
    // src/liboslexec/optexture.cpp:54-111); the file must have been
    // registered with oslg_texture_create. Options: wrap/swrap/twrap
    // (black, clamp, periodic, mirror; OIIO's default is black), width,
    // firstchannel.
    // gettextureinfo(filename, [s, t,] dataname, data) over the registered
    // textures (RendererServices::get_texture_info, rendservices.cpp:429-470,
    // answering from OpenImageIO's image info): the answer is known
    // when the group is lowered, so it becomes constants. A query whose data
    // has the wrong type, an unknown name, or a texture that is not
    // registered returns 0 and leaves data untouched, except "exists",
    // which always succeeds.
    bool lower_gettextureinfo(const LOp& op) {
        const size_t na = op.args.size();
        if (na != 4 && na != 6) return fail("gettextureinfo takes (filename, [s, t,] dataname, data)");
        const int fsym = op.args[1], nsym = op.args[na - 2], dsym = op.args[na - 1];
        if (!is_string(fsym) || !syms[fsym].is_const || !is_string(nsym) || !syms[nsym].is_const)
            return fail("gettextureinfo: the file and data names must be constant strings");
        const std::string file = const_string(fsym), what = const_string(nsym);
        const TypeSpec dt = syms[dsym].type;
        auto it = ss.texture_info.find(file);
        const TextureInfo* ti = it == ss.texture_info.end() ? nullptr : &it->second;
        std::vector<float> vals;
        std::vector<std::string> strs;
        bool ok = false;
        const bool is_int_arr = dt.base == BT_INT && dt.arraylen > 0;
        if (what == "exists" && dt.base == BT_INT && !dt.is_array()) {
            vals = { ti ? 1.0f : 0.0f };
            ok = true;
        } else if (ti) {
            const int w = ti->width, h = ti->height, nc = ti->nchannels;
            if (what == "resolution" && is_int_arr && (dt.arraylen == 2 || dt.arraylen == 3)) {
                vals = { (float)w, (float)h };
                if (dt.arraylen == 3) vals.push_back(1.0f);
                ok = true;
            } else if (what == "channels" && dt.base == BT_INT && !dt.is_array()) {
                vals = { (float)nc };
                ok = true;
            } else if ((what == "texturetype" || what == "textureformat") && dt.base == BT_STRING && !dt.is_array()) {
                strs = { "Plain Texture" };
                ok = true;
            } else if ((what == "datawindow" || what == "displaywindow") && is_int_arr
                       && (dt.arraylen == 4 || dt.arraylen == 6)) {
                vals = dt.arraylen == 4 ? std::vector<float>{ 0.0f, 0.0f, (float)(w - 1), (float)(h - 1) }
                                        : std::vector<float>{ 0.0f, 0.0f, 0.0f, (float)(w - 1), (float)(h - 1), 0.0f };
                ok = true;
            } else if ((what == "averagecolor" || (what == "constantcolor" && ti->constant)) && dt.base == BT_TRIPLE
                       && !dt.is_array()) {
                for (int c = 0; c < 3; ++c) vals.push_back(ti->average[(size_t)(nc >= 3 ? c : 0)]);
                ok = true;
            } else if ((what == "averagealpha" || (what == "constantalpha" && ti->constant)) && dt.base == BT_FLOAT
                       && !dt.is_array() && (nc == 4 || nc == 2)) {
                vals = { ti->average[(size_t)nc - 1] };
                ok = true;
            }
        }
        if (ok) {
            GSym c;
            c.name = "$texinfo";
            c.type = dt;
            c.kind = SK_CONST;
            c.is_const = true;
            c.cval = vals;
            c.sval = strs;
            const int cs = add_sym(c);
            syms[cs].slot = (int)pool_add(syms[cs]);
            const uint32_t el = (uint32_t)dt.elems();
            emit(OP_ASSIGN, { A(dsym), A(cs), el, el, el }, "gettextureinfo");
        }
        const int rc = const_int(ok ? 1 : 0);
        syms[rc].slot = (int)pool_add(syms[rc]);
        emit(OP_ASSIGN, { A(op.args[0]), A(rc), 1u, 1u, 1u }, "gettextureinfo");
        return true;
    }

    bool lower_texture(const LOp& op) {
        const size_t na = op.args.size();
        if (na < 4) return fail("texture needs a result, a file name and s, t");
        if (!is_string(op.args[1]) || !syms[op.args[1]].is_const)
            return fail("texture: the file name must be a constant string");
        const std::string fname = const_string(op.args[1]);
        auto it = ss.texture_ids.find(fname);
        if (it == ss.texture_ids.end()) return fail("texture '" + fname + "' is not registered");
        if (na > 4 && !is_string(op.args[4]))
            return fail("texture: explicit derivative arguments are not supported (the s, t derivatives are used)");
        uint32_t sw = TW_BLACK, tw = TW_BLACK;
        int first = 0;
        float width = 1.0f;
        for (size_t k = 4; k < na; k += 2) {
            if (k + 1 >= na || !is_string(op.args[k]) || !syms[op.args[k]].is_const)
                return fail("texture: options are constant name/value pairs");
            const std::string on = const_string(op.args[k]);
            const int v = op.args[k + 1];
            if (!syms[v].is_const) return fail("texture option '" + on + "' must be a constant");
            if (on == "wrap" || on == "swrap" || on == "twrap") {
                const std::string m = is_string(v) ? const_string(v) : std::string();
                uint32_t mode;
                if (m == "black" || m == "default") mode = TW_BLACK;
                else if (m == "clamp") mode = TW_CLAMP;
                else if (m == "periodic") mode = TW_PERIODIC;
                else if (m == "mirror") mode = TW_MIRROR;
                else return fail("texture: wrap mode '" + m + "' is not supported");
                if (on != "twrap") sw = mode;
                if (on != "swrap") tw = mode;
            } else if (on == "width" && !syms[v].cval.empty()) {
                width = syms[v].cval[0];
            } else if (on == "firstchannel" && !syms[v].cval.empty()) {
                first = (int)syms[v].cval[0];
                if (first < 0 || first > 255) return fail("texture: firstchannel out of range");
            } else {
                return fail("texture option '" + on + "' is not supported");
            }
        }
        if (it->second > 255) return fail("too many textures");
        const int wc = const_float(width);
        syms[wc].slot = (int)pool_add(syms[wc]);
        emit(OP_TEXTURE, { A(op.args[0]), A(op.args[2]), A(op.args[3]),
                           (uint32_t)it->second | (sw << 8) | (tw << 12) | ((uint32_t)first << 16), A(wc) }, "texture");
        return true;
    }

    // getattribute ([object,] name, [index,] dest) (osl_get_attribute,
    // src/liboslexec/opattribute.cpp; folding as constfold_getattribute,
    // src/liboslexec/constfold.cpp:2262-2360). The group's own names
    // (osl:version, shader:shadername, shader:layername, shader:groupname)
    // and the renderer's registered uniform attributes (the answers a
    // BatchedRendererServices gives for uniform attributes,
    // batched_rendererservices.h:118-170) become constants: `dest = value;
    // result = 1`. A name nobody answers for gives `result = 0` and leaves
    // dest unchanged, as the renderer's `false` does.
    int const_words(const TypeSpec& t, const std::vector<uint32_t>& w) {
        GSym d; d.name = "$attr"; d.type = t; d.kind = SK_CONST; d.is_const = true;
        int k = add_sym(d);
        syms[k].slot = (int)pool.size();
        pool.insert(pool.end(), w.begin(), w.end());
        return k;
    }
    // A per-point attribute of the shaded object: a userdata symloc with the
    // attribute's name and type (the renderer's per-point answer, read from
    // the userdata arena like an interpolated parameter). Looked up before
    // the scene-wide registered attributes, as the reference searches the
    // object first.
    bool load_userdata_attribute(const std::string& attr, int dest, int result) {
        const TypeSpec& dt = syms[dest].type;
        for (const SymLoc& sl : g.symlocs) {
            if (sl.arena != ARENA_USERDATA || sl.name != attr) continue;
            if (sl.type.base != dt.base || sl.type.arraylen != dt.arraylen || dt.is_array()
                || dt.base == BT_STRING || dt.base == BT_CLOSURE)
                return false;
            emit(OP_LOAD_USERDATA, { A(dest), (uint32_t)sl.offset, (uint32_t)sl.stride,
                                     (dt.base == BT_INT ? 1u : 0u) | (sl.derivs ? 2u : 0u) },
                 "getattribute");
            const int r = const_int(1);
            syms[r].slot = (int)pool_add(syms[r]);
            emit(OP_ASSIGN, { A(result), A(r), 1u, 1u, 1u }, "getattribute");
            return true;
        }
        return false;
    }
    bool lower_getattribute(const LOp& op) {
        const size_t na = op.args.size();
        if (na < 3 || na > 5) return fail("getattribute takes ([object,] name, [index,] value)");
        const bool array_lookup = na >= 4 && is_int(op.args[na - 2]);
        const bool object_lookup = na >= 4 && is_string(op.args[2]);
        const int name_sym = op.args[object_lookup ? 2 : 1];
        const int dest = op.args[na - 1];
        auto constant = [&](int s) { return syms[s].is_const; };
        if (!constant(name_sym) || (object_lookup && !constant(op.args[1]))
            || (array_lookup && !constant(op.args[na - 2])))
            return fail("getattribute: attribute names, object names and indices must be constants "
                        "(per-point attribute lookups are not supported)");
        const std::string attr = const_string(name_sym);
        const std::string object = object_lookup ? const_string(op.args[1]) : std::string();
        const TypeSpec& dt = syms[dest].type;
        std::vector<uint32_t> words;
        bool found = false;
        auto one_string = [&](const std::string& v) {
            if (dt.base == BT_STRING && !dt.is_array() && !array_lookup) {
                words = { string_hash(v) };
                found = true;
            }
        };
        const int li = op.layer >= 0 ? op.layer : 0;
        if (object.empty() && attr == "osl:version") {
            if (dt.base == BT_INT && !dt.is_array() && !array_lookup) {
                words = { (uint32_t)kOslVersionCode };
                found = true;
            }
        } else if (object.empty() && attr == "shader:shadername") {
            one_string(g.layers[li].master->name);
        } else if (object.empty() && attr == "shader:layername") {
            one_string(g.layers[li].layername);
        } else if (object.empty() && attr == "shader:groupname") {
            one_string(g.name);
        } else if (!object_lookup && !array_lookup && load_userdata_attribute(attr, dest, op.args[0])) {
            return true;
        } else {
            auto it = ss.attributes.find({ object, attr });
            if (it != ss.attributes.end()) {
                const RendererAttribute& ra = it->second;
                std::vector<uint32_t> rw = ra.words;
                if (ra.type.base == BT_STRING) {
                    rw.clear();
                    for (const std::string& x : ra.strings) rw.push_back(string_hash(x));
                }
                const bool same_elem = ra.type.base == dt.base;
                const size_t per = (size_t)ra.type.ncomp();
                if (array_lookup) {
                    const int idx = (int)syms[op.args[na - 2]].cval.at(0);
                    if (same_elem && ra.type.is_array() && !dt.is_array() && idx >= 0 && idx < ra.type.elems()
                        && rw.size() >= (size_t)(idx + 1) * per) {
                        words.assign(rw.begin() + (size_t)idx * per, rw.begin() + (size_t)(idx + 1) * per);
                        found = true;
                    }
                } else if (same_elem && ra.type.arraylen == dt.arraylen) {
                    words = rw;
                    found = true;
                }
            }
        }
        if (found) {
            const int c = const_words(dt, words);
            const uint32_t e = (uint32_t)dt.elems();
            emit(OP_ASSIGN, { A(dest), A(c), e, e, e }, "getattribute");
        }
        const int r = const_int(found ? 1 : 0);
        syms[r].slot = (int)pool_add(syms[r]);
        emit(OP_ASSIGN, { A(op.args[0]), A(r), 1u, 1u, 1u }, "getattribute");
        return true;
    }

    // ---- named coordinate systems ---------------------------------------------
    // Spaces resolve at lowering time to the renderer's registered uniform
    // matrices (oslg_renderer_matrix: RendererServices::get_matrix for named
    // spaces, and the object/shader to common transforms). "common" and its
    // synonym "world" are the identity (osl_get_matrix / osl_get_inverse_matrix,
    // src/liboslexec/opmatrix.cpp:141-196); inverses are taken in double
    // precision (a singular matrix inverts to the identity, as Imath's
    // non-throwing inverse does).
    using M44 = std::array<float, 16>;
    static M44 m_identity() {
        M44 m{};
        for (int i = 0; i < 4; ++i) m[(size_t)i * 5] = 1.0f;
        return m;
    }
    static M44 m_mul(const M44& A, const M44& B) {
        M44 c{};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j)
                c[(size_t)(i * 4 + j)] = A[(size_t)(i * 4 + 0)] * B[(size_t)(0 * 4 + j)]
                                       + A[(size_t)(i * 4 + 1)] * B[(size_t)(1 * 4 + j)]
                                       + A[(size_t)(i * 4 + 2)] * B[(size_t)(2 * 4 + j)]
                                       + A[(size_t)(i * 4 + 3)] * B[(size_t)(3 * 4 + j)];
        return c;
    }
    static M44 m_inverse(const M44& m) {
        double a[4][8];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 8; ++j) a[i][j] = j < 4 ? (double)m[(size_t)(i * 4 + j)] : (j - 4 == i ? 1.0 : 0.0);
        for (int c = 0; c < 4; ++c) {
            int piv = c;
            for (int r = c + 1; r < 4; ++r)
                if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
            if (a[piv][c] == 0.0) return m_identity();
            if (piv != c)
                for (int j = 0; j < 8; ++j) std::swap(a[c][j], a[piv][j]);
            const double d = a[c][c];
            for (int j = 0; j < 8; ++j) a[c][j] /= d;
            for (int r = 0; r < 4; ++r) {
                if (r == c || a[r][c] == 0.0) continue;
                const double f = a[r][c];
                for (int j = 0; j < 8; ++j) a[r][j] -= f * a[c][j];
            }
        }
        M44 inv{};
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) inv[(size_t)(i * 4 + j)] = (float)a[i][j + 4];
        return inv;
    }
    static std::string common_name(const std::string& s) { return s == "world" ? std::string("common") : s; }
    bool space_to_common(const std::string& sp, M44& M) const {
        if (sp == "common") { M = m_identity(); return true; }
        auto it = ss.named_matrices.find(sp);
        if (it == ss.named_matrices.end()) { M = m_identity(); return false; }
        M = it->second;
        return true;
    }
    // osl_get_from_to_matrix (opmatrix.cpp:231-240): get_matrix(from) *
    // get_inverse_matrix(to), an unknown space contributing the identity
    bool named_from_to(const LOp& op, int from_sym, int to_sym, M44& M, bool& ok) {
        if (!syms[from_sym].is_const || !syms[to_sym].is_const)
            return fail(op.name + ": space names must be constant strings");
        const std::string from = common_name(const_string(from_sym)), to = common_name(const_string(to_sym));
        M44 F, T;
        ok = space_to_common(from, F);
        ok = space_to_common(to, T) && ok;
        M = m_mul(F, to == "common" ? m_identity() : m_inverse(T));
        return true;
    }
    int const_matrix(const M44& M) {
        TypeSpec t;
        t.base = BT_MATRIX;
        std::vector<uint32_t> w(16);
        for (int i = 0; i < 16; ++i) std::memcpy(&w[(size_t)i], &M[(size_t)i], 4);
        return const_words(t, w);
    }
    // transform{,v,n} ([from,] to, p) (llvm_gen_transform,
    // src/liboslexec/llvm_gen.cpp:2025-2086; osl_transform_triple,
    // opmatrix.cpp:244-300): the same space twice copies p; an unknown space
    // copies p as well (the reference also reports it as an error).
    // A colour space name the colour system knows (ColorSystem::transformc,
    // src/liboslexec/opcolor.cpp:324-380; the system's own colour space
    // is rgb); -1 for spaces only OpenColorIO could convert.
    int color_space_code(const std::string& s) const {
        if (s == "rgb" || s == "RGB" || s == "linear" || s == ss.opts.colorspace) return CS_RGB;
        if (s == "hsv") return CS_HSV;
        if (s == "hsl") return CS_HSL;
        if (s == "YIQ") return CS_YIQ;
        if (s == "XYZ") return CS_XYZ;
        if (s == "xyY") return CS_XYY;
        if (s == "sRGB") return CS_SRGB;
        return -1;
    }
    // r = C converted from space `from` (gsym, -1: rgb) to `to` (-1: rgb)
    bool lower_color_transform(int r, int c, int from, int to) {
        auto code = [&](int gs, int& out) {
            if (gs < 0) { out = CS_RGB; return true; }
            if (!syms[gs].is_const) return fail("transformc: colour space names must be constant strings");
            out = color_space_code(const_string(gs));
            if (out < 0) return fail("colour space '" + const_string(gs) + "' needs OpenColorIO, which is not supported");
            return true;
        };
        int f, t;
        if (!code(from, f) || !code(to, t)) return false;
        const ColorSys& cs = csys();
        std::vector<float> tab;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) tab.push_back(cs.xyz2rgb[i][j]);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) tab.push_back(cs.rgb2xyz[i][j]);
        emit(OP_TRANSFORMC, { A(r), A(c), (uint32_t)f | ((uint32_t)t << 8), A(const_floats(tab)) }, "transformc");
        return true;
    }

    bool lower_named_transform(const LOp& op) {
        const std::string& n = op.name;
        const size_t na = op.args.size();
        if (na != 3 && na != 4) return fail(n + " takes ([from,] to, p) or (M, p)");
        const int p = op.args[na - 1];
        const int to = op.args[na - 2];
        if (!is_string(to) || (na == 4 && !is_string(op.args[1]))) return fail(n + ": bad space arguments");
        if (!syms[to].is_const || (na == 4 && !syms[op.args[1]].is_const))
            return fail(n + ": space names must be constant strings");
        const std::string from_s = na == 4 ? common_name(const_string(op.args[1])) : std::string("common");
        const std::string to_s = common_name(const_string(to));
        M44 F, T;
        bool ok = space_to_common(from_s, F);
        ok = space_to_common(to_s, T) && ok;
        if (from_s == to_s || !ok) {
            emit(OP_ASSIGN, { A(op.args[0]), A(p), 1u, 1u, 1u }, n);
            return true;
        }
        const M44 M = from_s == "common" ? m_inverse(T) : to_s == "common" ? F : m_mul(F, m_inverse(T));
        const uint32_t kind = n == "transform" ? 0u : n == "transformv" ? 1u : 2u;
        emit(OP_TRANSFORM, { A(op.args[0]), A(p), A(const_matrix(M)), kind }, n);
        return true;
    }

    // environment r filename R ["option", value]... (osl_environment,
    // src/liboslexec/optexture.cpp): the registered image is a
    // latitude-longitude map (z up); options width, firstchannel.
    bool lower_environment(const LOp& op) {
        const size_t na = op.args.size();
        if (na < 3) return fail("environment needs a result, a file name and a direction");
        if (!is_string(op.args[1]) || !syms[op.args[1]].is_const)
            return fail("environment: the file name must be a constant string");
        if (!is_triple(op.args[2])) return fail("environment: the direction must be a vector");
        const std::string fname = const_string(op.args[1]);
        auto it = ss.texture_ids.find(fname);
        if (it == ss.texture_ids.end()) return fail("environment map '" + fname + "' is not registered");
        if (na > 3 && !is_string(op.args[3]))
            return fail("environment: explicit derivative arguments are not supported (those of R are used)");
        int first = 0;
        float width = 1.0f;
        for (size_t k = 3; k < na; k += 2) {
            if (k + 1 >= na || !is_string(op.args[k]) || !syms[op.args[k]].is_const)
                return fail("environment: options are constant name/value pairs");
            const std::string on = const_string(op.args[k]);
            const int v = op.args[k + 1];
            if (!syms[v].is_const || syms[v].cval.empty())
                return fail("environment option '" + on + "' must be a numeric constant");
            if (on == "width") width = syms[v].cval[0];
            else if (on == "firstchannel") first = (int)syms[v].cval[0];
            else return fail("environment option '" + on + "' is not supported");
            if (first < 0 || first > 255) return fail("environment: firstchannel out of range");
        }
        if (it->second > 255) return fail("too many textures");
        const int wc = const_float(width);
        syms[wc].slot = (int)pool_add(syms[wc]);
        emit(OP_ENVIRONMENT, { A(op.args[0]), A(op.args[2]), 0u, (uint32_t)it->second | ((uint32_t)first << 16), A(wc) },
             "environment");
        return true;
    }

    bool lower_op(const LOp& op, int depth, int loopl) {
        const std::string& n = op.name;
        auto a = [&](int i) { return A(op.args[i]); };
        size_t na = op.args.size();
        if (n == "nop" || n == "useparam" || n == "end") return true;
        if (n == "break") { emit(OP_BREAK, { 0u, 0u, 0u, (uint32_t)loopl }, n); return true; }
        if (n == "continue") { emit(OP_CONTINUE, { 0u, 0u, 0u, (uint32_t)loopl }, n); return true; }
        if (n == "return") { emit(OP_RETURN, {}, n); return true; }
        if (n == "exit") { emit(OP_EXIT, {}, n); return true; }
        if (n == "__layer_end") { emit(OP_LAYER_END, {}, "layer"); return true; }
        if (n == "__store_heap") {
            emit(OP_STORE_HEAP, { a(0), (uint32_t)op.imm[0], (uint32_t)op.imm[1] }, "symbol");
            return true;
        }
        if (n == "__stores_end") { emit(OP_STORES_END, { (uint32_t)op.imm[0] }, "layer"); return true; }
        if (n == "__load_userdata") {
            int s = op.args[0];
            emit(OP_LOAD_USERDATA, { a(0), (uint32_t)op.imm[0], (uint32_t)op.imm[1],
                                     (is_int(s) ? 1u : 0u) | (op.imm[2] ? 2u : 0u) },
                 "userdata");
            return true;
        }
        if (n == "__cl_node") {
            // a closure op whose node sits at a fixed heap slot (static closures)
            size_t ni = 1;
            int weight = -1;
            if (na > 1 && !is_string(op.args[1])) { weight = op.args[1]; ni = 2; }
            std::string cname = const_string(op.args[ni]);
            auto it = ss.closure_ids.find(cname);
            if (it == ss.closure_ids.end()) return fail("closure '" + cname + "' is not registered");
            if (!closure_params_complete(cname, op)) return false;
            std::vector<uint32_t> params;
            for (size_t i = ni + 1; i < na && params.size() < 11; ++i) params.push_back(A(op.args[i]));
            while (params.size() < 11) params.push_back(kNoArg);
            emit(OP_CLOSURE_NODE, { A(op.args[0]), (uint32_t)it->second, weight >= 0 ? A(weight) : kNoArg, params[0],
                                    params[1], params[2], params[3] },
                 "closure");
            if (na > ni + 5)
                emit(OP_NOP, { params[4], params[5], params[6], params[7], params[8], params[9], params[10] },
                     "closure-params");
            return true;
        }
        if (n == "__cl_mulnode") {
            // cw = (MUL weight product) * the component's own weight (node words 1..3)
            const uint32_t nw = arg_make((uint32_t)syms[op.args[2]].slot + 1u, false, false, TC_TRIPLE);
            emit(OP_MUL, { a(0), a(1), nw }, "closure-weight");
            return true;
        }
        if (n == "__cl_store" || n == "__cl_bsdf_eval" || n == "__cl_bsdf_sample") {
            const size_t fixed = n == "__cl_store" ? 0 : (n == "__cl_bsdf_eval" ? 2 : 1);
            const uint32_t nterms = (uint32_t)((na - fixed) / 3);
            if (n == "__cl_store")
                emit(OP_CL_STORE, { nterms, (uint32_t)op.imm[0], (uint32_t)op.imm[1], (uint32_t)op.imm[3] }, "output");
            else if (n == "__cl_bsdf_eval")
                emit(OP_CL_BSDF_EVAL, { nterms, (uint32_t)op.imm[0], (uint32_t)op.imm[1], a(0), a(1), string_hash("ggx") },
                     "bsdf_eval");
            else
                emit(OP_CL_BSDF_SAMPLE, { nterms, (uint32_t)op.imm[0], (uint32_t)op.imm[1], a(0), string_hash("ggx"),
                                          (uint32_t)op.imm[2], (uint32_t)op.imm[3] },
                     "bsdf_sample");
            // the term table: {node slot, weight operand, presence operand}, two per carrier
            for (uint32_t j = 0; j < nterms; j += 2) {
                uint32_t w[6] = { 0u, kNoArg, kNoArg, 0u, kNoArg, kNoArg };
                for (uint32_t t = 0; t < 2 && j + t < nterms; ++t) {
                    const size_t b = fixed + 3 * (j + t);
                    w[3 * t + 0] = (uint32_t)syms[op.args[b]].slot;
                    w[3 * t + 1] = op.args[b + 1] == none_sym ? kNoArg : A(op.args[b + 1]);
                    w[3 * t + 2] = op.args[b + 2] == none_sym ? kNoArg : A(op.args[b + 2]);
                }
                emit(OP_NOP, { w[0], w[1], w[2], w[3], w[4], w[5], 0u }, "closure-terms");
            }
            return true;
        }
        if (n == "__bsdf_eval") {
            // renderer-side evaluation of a closure output (testrender's
            // CompositeBSDF::eval, src/testrender/shading.h:364-374)
            uses_closures = true;
            emit(OP_BSDF_EVAL, { a(0), (uint32_t)op.imm[0], (uint32_t)op.imm[1], a(1), a(2), string_hash("ggx") },
                 "bsdf_eval");
            return true;
        }
        if (n == "__bsdf_sample") {
            // renderer-side sampling of a closure output (testrender's
            // CompositeBSDF::prepare + sample, src/testrender/shading.h:322-398)
            uses_closures = true;
            emit(OP_BSDF_SAMPLE, { a(0), (uint32_t)op.imm[0], (uint32_t)op.imm[1], a(1), string_hash("ggx"),
                                   (uint32_t)op.imm[2], (uint32_t)op.imm[3] },
                 "bsdf_sample");
            return true;
        }
        if (n == "__store_output") {
            int s = op.args[0];
            if (is_closure(s)) {
                emit(OP_STORE_CLOSURE, { a(0), (uint32_t)op.imm[0], (uint32_t)op.imm[1], (uint32_t)op.imm[3] },
                     "output");
                return true;
            }
            uint32_t flags = (op.imm[2] ? 1u : 0u) | (is_int(s) ? 2u : 0u);
            emit(OP_STORE_OUTPUT, { a(0), (uint32_t)op.imm[0], (uint32_t)op.imm[1], flags,
                                    (uint32_t)syms[s].type.elems() },
                 "output");
            return true;
        }
        if (n == "assign") {
            if (na < 2) return fail("assign needs 2 args");
            int r = op.args[0], s = op.args[1];
            if (is_closure(r)) {
                emit(OP_ASSIGN, { a(0), a(1), (uint32_t)syms[r].type.elems() }, n);
                return true;
            }
            emit(OP_ASSIGN, { a(0), a(1), (uint32_t)std::min(syms[r].type.elems(), syms[s].type.elems()),
                              (uint32_t)syms[r].type.elems(), (uint32_t)syms[s].type.elems() },
                 n);
            return true;
        }
        static const std::map<std::string, std::pair<uint16_t, uint16_t>> arith = {
            { "add", { OP_ADD, OP_IADD } }, { "sub", { OP_SUB, OP_ISUB } },
            { "mul", { OP_MUL, OP_IMUL } }, { "div", { OP_DIV, OP_IDIV } },
            { "mod", { OP_MOD, OP_IMOD } } };
        auto ar = arith.find(n);
        if (ar != arith.end()) {
            if (na < 3) return fail(n + " needs 3 args");
            int r = op.args[0], x = op.args[1], y = op.args[2];
            if (is_closure(r)) {
                uses_closures = true;
                if (n == "add") { emit(OP_CLOSURE_ADD, { a(0), a(1), a(2) }, n); return true; }
                if (n == "mul") {
                    if (is_closure(x)) emit(OP_CLOSURE_MUL, { a(0), a(1), a(2) }, n);
                    else emit(OP_CLOSURE_MUL, { a(0), a(2), a(1) }, n);
                    return true;
                }
                return fail("closure " + n + " is not an OSL operation");
            }
            if (is_int(r) && is_int(x) && is_int(y)) {
                emit(ar->second.second, { a(0), a(1), a(2) }, n);
                return true;
            }
            if ((n == "mul" || n == "div") && is_matrix(r) && (is_matrix(x) || is_matrix(y) || n == "div")) {
                emit(n == "mul" ? OP_MMUL : OP_MDIV, { a(0), a(1), a(2) }, n);
                return true;
            }
            emit(ar->second.first, { a(0), a(1), a(2) }, n);
            return true;
        }
        if (n == "neg") {
            emit(is_int(op.args[0]) ? OP_INEG : OP_NEG, { a(0), a(1) }, n);
            return true;
        }
        static const std::map<std::string, uint16_t> cmp = {
            { "eq", OP_EQ }, { "neq", OP_NEQ }, { "lt", OP_LT }, { "gt", OP_GT }, { "le", OP_LE },
            { "ge", OP_GE }, { "and", OP_AND }, { "or", OP_OR }, { "bitand", OP_BITAND },
            { "bitor", OP_BITOR }, { "xor", OP_XOR }, { "shl", OP_SHL }, { "shr", OP_SHR } };
        auto cm = cmp.find(n);
        if (cm != cmp.end()) {
            if (na < 3) return fail(n + " needs 3 args");
            emit(cm->second, { a(0), a(1), a(2) }, n);
            return true;
        }
        if (n == "compl") { emit(OP_COMPL, { a(0), a(1) }, n); return true; }
        static const std::map<std::string, uint16_t> unary = {
            { "floor", OP_FLOOR }, { "ceil", OP_CEIL }, { "round", OP_ROUND }, { "trunc", OP_TRUNC },
            { "sign", OP_SIGN }, { "sqrt", OP_SQRT }, { "inversesqrt", OP_INVSQRT },
            { "cbrt", OP_CBRT }, { "sin", OP_SIN }, { "cos", OP_COS }, { "tan", OP_TAN },
            { "asin", OP_ASIN }, { "acos", OP_ACOS }, { "atan", OP_ATAN }, { "sinh", OP_SINH },
            { "cosh", OP_COSH }, { "tanh", OP_TANH }, { "exp", OP_EXP }, { "exp2", OP_EXP2 },
            { "expm1", OP_EXPM1 }, { "log", OP_LOG }, { "log2", OP_LOG2 }, { "log10", OP_LOG10 },
            { "radians", OP_RADIANS }, { "degrees", OP_DEGREES }, { "isnan", OP_ISNAN },
            { "isinf", OP_ISINF }, { "isfinite", OP_ISFINITE }, { "logb", OP_LOGB }, { "erf", OP_ERF },
            { "erfc", OP_ERFC } };
        if (n == "abs" || n == "fabs") {
            emit(is_int(op.args[0]) ? OP_IABS : OP_ABS, { a(0), a(1) }, n);
            return true;
        }
        // ops the reference's default build computes with OpenImageIO's fast_*
        // functions (wide_optranscendental.cpp:34-66, wide_optrigonometric.cpp:16-47)
        static const std::set<uint16_t> fast_ops = { OP_SIN, OP_COS, OP_TAN, OP_ASIN, OP_ACOS, OP_ATAN,
                                                     OP_SINH, OP_COSH, OP_TANH, OP_EXP, OP_EXP2, OP_EXPM1,
                                                     OP_LOG, OP_LOG2, OP_LOG10, OP_ERF, OP_ERFC, OP_CBRT };
        const uint32_t fast = ss.opts.fast_math ? 1u : 0u;
        auto un = unary.find(n);
        if (un != unary.end()) {
            if (na < 2) return fail(n + " needs 2 args");
            emit(un->second, { a(0), a(1), fast_ops.count(un->second) ? fast : 0u }, n);
            return true;
        }
        if (n == "pow" || n == "atan2" || n == "fmod") {
            emit(n == "pow" ? OP_POW : n == "atan2" ? OP_ATAN2 : OP_FMOD, { a(0), a(1), a(2), n == "fmod" ? 0u : fast },
                 n);
            return true;
        }
        if (n == "min" || n == "max") {
            bool ints = is_int(op.args[0]);
            emit(n == "min" ? (ints ? OP_IMIN : OP_MIN) : (ints ? OP_IMAX : OP_MAX), { a(0), a(1), a(2) }, n);
            return true;
        }
        if (n == "clamp") { emit(OP_CLAMP, { a(0), a(1), a(2), a(3) }, n); return true; }
        if (n == "mix") { emit(OP_MIX, { a(0), a(1), a(2), a(3) }, n); return true; }
        if (n == "select") { emit(OP_SELECT, { a(0), a(1), a(2), a(3) }, n); return true; }
        if (n == "step") { emit(OP_STEP, { a(0), a(1), a(2) }, n); return true; }
        if (n == "smoothstep") { emit(OP_SMOOTHSTEP, { a(0), a(1), a(2), a(3) }, n); return true; }
        if (n == "dot") { emit(OP_DOT, { a(0), a(1), a(2) }, n); return true; }
        if (n == "cross") { emit(OP_CROSS, { a(0), a(1), a(2) }, n); return true; }
        if (n == "length") { emit(OP_LENGTH, { a(0), a(1) }, n); return true; }
        if (n == "normalize") { emit(OP_NORMALIZE, { a(0), a(1) }, n); return true; }
        if (n == "distance") { emit(OP_DISTANCE, { a(0), a(1), a(2) }, n); return true; }
        if (n == "Dx") { emit(OP_DX, { a(0), a(1) }, n); return true; }
        if (n == "Dy") { emit(OP_DY, { a(0), a(1) }, n); return true; }
        if (n == "area") { emit(OP_AREA, { a(0), a(1) }, n); return true; }
        if (n == "filterwidth") { emit(OP_FILTERWIDTH, { a(0), a(1) }, n); return true; }
        if (n == "compref") { emit(OP_COMPREF, { a(0), a(1), a(2) }, n); return true; }
        if (n == "compassign") { emit(OP_COMPASSIGN, { a(0), a(1), a(2) }, n); return true; }
        if (n == "mxcompref") { emit(OP_MXCOMPREF, { a(0), a(1), a(2), a(3) }, n); return true; }
        if (n == "mxcompassign") { emit(OP_MXCOMPASSIGN, { a(0), a(1), a(2), a(3) }, n); return true; }
        if (n == "aref") {
            emit(OP_AREF, { a(0), a(1), a(2), (uint32_t)syms[op.args[1]].type.elems() }, n);
            return true;
        }
        if (n == "aassign") {
            emit(OP_AASSIGN, { a(0), a(1), a(2), (uint32_t)syms[op.args[0]].type.elems() }, n);
            return true;
        }
        if (n == "arraycopy") {  // batched_llvm_gen.cpp:2257-2264: an assignment
            emit(OP_ASSIGN, { a(0), a(1), (uint32_t)std::min(syms[op.args[0]].type.elems(), syms[op.args[1]].type.elems()),
                              (uint32_t)syms[op.args[0]].type.elems(), (uint32_t)syms[op.args[1]].type.elems() },
                 n);
            return true;
        }
        if (n == "sincos") { emit(OP_SINCOS, { a(0), a(1), a(2), ss.opts.fast_math ? 1u : 0u }, n); return true; }
        if (n == "calculatenormal") { emit(OP_CALCNORMAL, { a(0), a(1) }, n); return true; }
        if (n == "backfacing") { emit(OP_LOAD_GLOBAL, { a(0), (uint32_t)G_BACKFACING }, n); return true; }
        if (n == "surfacearea") { emit(OP_LOAD_GLOBAL, { a(0), (uint32_t)G_SURFACEAREA }, n); return true; }
        if (n == "trace") {
            // RendererServices::trace (rendservices.cpp:511-517): the default
            // renderer services trace nothing and report no hit; a sourced
            // getmessage("trace", ...) then finds nothing either
            const int c = const_int(0);
            syms[c].slot = (int)pool_add(syms[c]);
            emit(OP_ASSIGN, { a(0), A(c), 1u, 1u, 1u }, n);
            return true;
        }
        if (n == "isconstant") {
            // what folding did not turn into 1 is not constant
            // (batched_llvm_gen.cpp:8079-8092)
            const int c = const_int(syms[op.args[1]].is_const ? 1 : 0);
            syms[c].slot = (int)pool_add(syms[c]);
            emit(OP_ASSIGN, { a(0), A(c), 1u, 1u, 1u }, n);
            return true;
        }
        if (n == "raytype") {
            // batched_llvm_gen.cpp:8520-8560: a constant name's bit is known
            // here; a varying name is looked up in the raytypes list
            const std::vector<std::string>& rt = ss.opts.raytypes;
            std::vector<float> hashes;
            if (is_string(op.args[1]) && syms[op.args[1]].is_const) {
                const std::string nm = const_string(op.args[1]);
                uint32_t bit = 0;
                for (size_t i = 0; i < rt.size() && i < 32; ++i)
                    if (rt[i] == nm) { bit = 1u << i; break; }
                emit(OP_RAYTYPE, { a(0), kNoArg, bit, kNoArg, 0u }, n);
                return true;
            }
            GSym t;
            t.name = "$raytypes"; t.type.base = BT_STRING; t.type.arraylen = (int)std::max<size_t>(1, rt.size());
            t.kind = SK_CONST; t.is_const = true; t.sval = rt;
            const int ts = add_sym(t);
            syms[ts].slot = (int)pool_add(syms[ts]);
            emit(OP_RAYTYPE, { a(0), a(1), 0u, A(ts), (uint32_t)std::min<size_t>(rt.size(), 32) }, n);
            return true;
        }
        if (n == "arraylength") {
            int c = const_int(syms[op.args[1]].type.elems());
            syms[c].slot = (int)pool_add(syms[c]);
            emit(OP_ASSIGN, { a(0), A(c), 1u, 1u, 1u }, n);
            return true;
        }
        if (n == "point" || n == "vector" || n == "normal" || n == "color") {
            if (na == 4) { emit(OP_CONSTRUCT3, { a(0), a(1), a(2), a(3) }, n); return true; }
            if (na == 2) { emit(OP_ASSIGN, { a(0), a(1), 1u, 1u, 1u }, n); return true; }
            if (na == 5 && is_string(op.args[1])) {
                // constructors in a named space: the triple, then from that
                // space to rgb (osl_prepend_color_from) or to "common"
                // (osl_prepend_point_from and its vector/normal forms)
                emit(OP_CONSTRUCT3, { a(0), a(2), a(3), a(4) }, n);
                if (n == "color") return lower_color_transform(op.args[0], op.args[0], op.args[1], -1);
                LOp t;
                t.name = n == "point" ? "transform" : n == "vector" ? "transformv" : "transformn";
                GSym c;
                c.name = "$space";
                c.type.base = BT_STRING;
                c.kind = SK_CONST;
                c.is_const = true;
                c.sval = { "common" };
                t.args = { op.args[0], op.args[1], add_sym(c), op.args[0] };
                return lower_named_transform(t);
            }
            return fail(n + ": unsupported constructor form");
        }
        if (n == "transformc") {  // transformc r [from] to C
            if (na == 3) return lower_color_transform(op.args[0], op.args[2], -1, op.args[1]);
            if (na == 4) return lower_color_transform(op.args[0], op.args[3], op.args[1], op.args[2]);
            return fail("transformc takes ([from,] to, color)");
        }
        if (n == "wavelength_color") {
            std::vector<float> t;
            const ColorSys& cs = csys();
            for (int i = 0; i < 3; ++i)
                for (int j = 0; j < 3; ++j) t.push_back(cs.xyz2rgb[i][j]);
            for (int i = 0; i < 81; ++i)
                for (int j = 0; j < 3; ++j) t.push_back(kCIE[i][j]);
            emit(OP_WAVELENGTH, { a(0), a(1), A(const_floats(t)) }, n);
            return true;
        }
        if (n == "matrix") {
            int r = op.args[0];
            if (na == 2 && !is_string(op.args[1])) {
                emit(OP_MATRIX_DIAG, { a(0), a(1) }, n);
                return true;
            }
            if (na == 3 && is_string(op.args[1]) && is_string(op.args[2])) {  // matrix(from, to)
                M44 M;
                bool ok;
                if (!named_from_to(op, op.args[1], op.args[2], M, ok)) return false;
                emit(OP_ASSIGN, { a(0), A(const_matrix(M)), 1u, 1u, 1u }, n);
                return true;
            }
            if ((na == 3 || na == 18) && is_string(op.args[1])) {
                // matrix(space, f) / matrix(space, 16 floats): the values,
                // then prepended by the space's matrix (osl_prepend_matrix_from,
                // src/liboslexec/opmatrix.cpp:210-229); an unknown space
                // leaves the values
                if (!syms[op.args[1]].is_const) return fail("matrix: the space name must be a constant string");
                if (na == 3) {
                    emit(OP_MATRIX_DIAG, { a(0), a(2) }, n);
                } else {
                    int zero = const_float(0.0f);
                    syms[zero].slot = (int)pool_add(syms[zero]);
                    emit(OP_MATRIX_DIAG, { a(0), A(zero) }, n);
                    for (int i = 0; i < 16; ++i) {
                        int ri = const_int(i / 4), ci = const_int(i % 4);
                        syms[ri].slot = (int)pool_add(syms[ri]);
                        syms[ci].slot = (int)pool_add(syms[ci]);
                        emit(OP_MXCOMPASSIGN, { A(r), A(ri), A(ci), a(2 + i) }, n);
                    }
                }
                M44 Mf;
                if (space_to_common(common_name(const_string(op.args[1])), Mf))
                    emit(OP_MMUL, { a(0), A(const_matrix(Mf)), a(0) }, n);
                return true;
            }
            if (na == 17) {
                int zero = const_float(0.0f);
                syms[zero].slot = (int)pool_add(syms[zero]);
                emit(OP_MATRIX_DIAG, { a(0), A(zero) }, n);
                for (int i = 0; i < 16; ++i) {
                    int ri = const_int(i / 4), ci = const_int(i % 4);
                    syms[ri].slot = (int)pool_add(syms[ri]);
                    syms[ci].slot = (int)pool_add(syms[ci]);
                    emit(OP_MXCOMPASSIGN, { A(r), A(ri), A(ci), a(1 + i) }, n);
                }
                return true;
            }
            return fail("matrix construction from named spaces is not supported yet");
        }
        if (n == "transpose") { emit(OP_TRANSPOSE, { a(0), a(1) }, n); return true; }
        if (n == "determinant") { emit(OP_DETERMINANT, { a(0), a(1) }, n); return true; }
        if (n == "transform" || n == "transformv" || n == "transformn") {
            // transform r M p  (matrix form)
            if (na == 3 && is_matrix(op.args[1])) {
                uint32_t kind = n == "transform" ? 0u : n == "transformv" ? 1u : 2u;
                if (n == "transform" && syms[op.args[2]].type.vecsem == VS_VECTOR) kind = 1u;
                if (n == "transform" && syms[op.args[2]].type.vecsem == VS_NORMAL) kind = 2u;
                emit(OP_TRANSFORM, { a(0), a(2), a(1), kind }, n);
                return true;
            }
            return lower_named_transform(op);
        }
        if (n == "getmatrix") {
            if (na != 4) return fail("getmatrix takes (from, to, M)");
            M44 M;
            bool ok;
            if (!named_from_to(op, op.args[1], op.args[2], M, ok)) return false;
            const int c = const_matrix(M);
            emit(OP_ASSIGN, { a(3), A(c), 1u, 1u, 1u }, n);
            const int r = const_int(ok ? 1 : 0);
            syms[r].slot = (int)pool_add(syms[r]);
            emit(OP_ASSIGN, { a(0), A(r), 1u, 1u, 1u }, n);
            return true;
        }
        if (n == "noise" || n == "snoise" || n == "pnoise" || n == "psnoise" || n == "cellnoise"
            || n == "hashnoise")
            return lower_noise(op);
        if (n == "hash") {
            emit(OP_HASH, { a(0), a(1), na > 2 ? a(2) : kNoArg }, n);
            return true;
        }
        if (n == "spline") {
            // spline r basis x [nknots] knots  (src/liboslexec/opspline.cpp)
            if (na < 4) return fail("spline needs at least 4 args");
            std::string basis = const_string(op.args[1]);
            static const std::map<std::string, int> bases = { { "catmull-rom", 0 }, { "bezier", 1 },
                                                              { "bspline", 2 }, { "hermite", 3 },
                                                              { "linear", 4 }, { "constant", 5 } };
            auto bi = bases.find(basis);
            if (bi == bases.end()) return fail("unknown spline basis '" + basis + "'");
            int knots = op.args[na - 1];
            int nknots_sym = na == 5 ? op.args[3] : -1;
            uint32_t nk = nknots_sym >= 0 ? A(nknots_sym) : kNoArg;
            emit(OP_SPLINE, { a(0), a(2), A(knots), (uint32_t)bi->second, nk,
                              (uint32_t)syms[knots].type.elems() },
                 n);
            return true;
        }
        if (n == "splineinverse") {
            // splineinverse r basis y [nknots] knots (float knots only), as
            // src/liboslexec/opspline.cpp:115-153
            if (na < 4) return fail("splineinverse needs at least 4 args");
            std::string basis = const_string(op.args[1]);
            static const std::map<std::string, int> bases = { { "catmull-rom", 0 }, { "bezier", 1 },
                                                              { "bspline", 2 }, { "hermite", 3 },
                                                              { "linear", 4 }, { "constant", 5 } };
            auto bi = bases.find(basis);
            if (bi == bases.end()) return fail("unknown spline basis '" + basis + "'");
            int knots = op.args[na - 1];
            if (syms[knots].type.base != BT_FLOAT || syms[op.args[0]].type.base != BT_FLOAT
                || syms[op.args[2]].type.base != BT_FLOAT)
                return fail("splineinverse takes and returns floats, with float knots");
            uint32_t nk = na == 5 ? A(op.args[3]) : kNoArg;
            emit(OP_SPLINEINV, { a(0), a(2), A(knots), (uint32_t)bi->second, nk,
                                 (uint32_t)syms[knots].type.elems() },
                 n);
            return true;
        }
        if (n == "blackbody") {
            const std::vector<float>& t = blackbody_pool();
            int tb = const_floats(t);
            emit(OP_BLACKBODY, { a(0), a(1), A(tb), (uint32_t)((t.size() - 9 - 243) / 3) }, n);
            return true;
        }
        if (n == "gettextureinfo") return lower_gettextureinfo(op);
        if (n == "texture") return lower_texture(op);
        if (n == "environment") return lower_environment(op);
        if (n == "getattribute") return lower_getattribute(op);
        if (n == "setmessage") {
            const TypeSpec& t = syms[op.args[1]].type;
            const uint32_t nw = (uint32_t)(t.ncomp() * t.elems());
            if (nw > 0xFFFFu || op.imm[0] > 0x7FFF) return fail("setmessage: value too large");
            emit(OP_SETMESSAGE, { a(2), a(3), a(1), nw | ((uint32_t)op.imm[0] << 16) }, n);
            return true;
        }
        if (n == "getmessage") {
            const TypeSpec& t = syms[op.args[2]].type;
            const uint32_t nw = (uint32_t)(t.ncomp() * t.elems());
            if (nw > 0xFFFFu || op.imm[0] > 0x7FFF) return fail("getmessage: value too large");
            emit(OP_GETMESSAGE, { a(0), a(3), a(4), a(2),
                                  nw | ((uint32_t)op.imm[0] << 16) | (ss.opts.strict_messages ? 0x80000000u : 0u) },
                 n);
            return true;
        }
        if (n == "luminance") {
            int sc = const_triple(luminance_scale());
            emit(OP_LUMINANCE, { a(0), a(1), A(sc) }, n);
            return true;
        }
        if (n == "closure") {
            // closure r [weight] name args...   (llvm_gen_closure, batched_llvm_gen.cpp:7310)
            uses_closures = true;
            if (closure_param_words(op) > kRecordParams) wide_nodes = true;
            size_t ni = 1;
            int weight = -1;
            if (na > 1 && !is_string(op.args[1])) { weight = op.args[1]; ni = 2; }
            std::string cname = const_string(op.args[ni]);
            auto it = ss.closure_ids.find(cname);
            if (it == ss.closure_ids.end()) return fail("closure '" + cname + "' is not registered");
            if (!closure_params_complete(cname, op)) return false;
            std::vector<uint32_t> params;
            for (size_t i = ni + 1; i < na && params.size() < 11; ++i) params.push_back(A(op.args[i]));
            while (params.size() < 11) params.push_back(kNoArg);
            emit(OP_CLOSURE, { a(0), (uint32_t)it->second, weight >= 0 ? A(weight) : kNoArg, params[0], params[1],
                               params[2], params[3] },
                 n);
            if (na > ni + 5)
                emit(OP_NOP, { params[4], params[5], params[6], params[7], params[8], params[9], params[10] },
                     "closure-params");
            return true;
        }
        return fail("op '" + n + "' is not supported by this executor");
    }

    // Interpreter feature tier the program needs (oslg_exec.h TierFns):
    // bit 0 noise/hash, bit 1 closures/BSDF/spline, bit 2 math/vector/matrix.
    uint32_t program_tier() const {
        uint32_t t = 0;
        for (const Op& op : ops) {
            switch (op.code) {
            case OP_NOISE: case OP_HASH: case OP_GABOR: t |= 1u; break;
            case OP_CLOSURE: case OP_CLOSURE_MUL: case OP_CLOSURE_ADD: case OP_STORE_CLOSURE: case OP_BSDF_EVAL:
            case OP_BSDF_SAMPLE: case OP_CLOSURE_NODE: case OP_CL_STORE: case OP_CL_BSDF_EVAL: case OP_CL_BSDF_SAMPLE:
            case OP_SPLINE: case OP_SPLINEINV:
                t |= 2u;
                break;
            case OP_CBRT: case OP_SIN: case OP_COS: case OP_TAN: case OP_ASIN: case OP_ACOS: case OP_ATAN:
            case OP_SINH: case OP_COSH: case OP_TANH: case OP_EXP: case OP_EXP2: case OP_EXPM1: case OP_LOG:
            case OP_LOG2: case OP_LOG10: case OP_POW: case OP_ATAN2: case OP_FMOD: case OP_CLAMP: case OP_MIX:
            case OP_SMOOTHSTEP: case OP_SELECT: case OP_DOT: case OP_CROSS: case OP_LENGTH: case OP_DISTANCE:
            case OP_NORMALIZE: case OP_TRANSFORM: case OP_MMUL: case OP_AREF: case OP_AASSIGN:
            case OP_MDIV: case OP_TRANSPOSE: case OP_DETERMINANT: case OP_AREA: case OP_FILTERWIDTH:
            case OP_LUMINANCE: case OP_BLACKBODY: case OP_TEXTURE: case OP_SETMESSAGE: case OP_GETMESSAGE:
            case OP_TRANSFORMC: case OP_WAVELENGTH:
            case OP_LOGB: case OP_ERF: case OP_ERFC: case OP_SINCOS: case OP_CALCNORMAL: case OP_RAYTYPE:
            case OP_ENVIRONMENT:
                t |= 4u;
                break;
            default: break;
            }
        }
        return t;
    }

    // isconnected(x) as RuntimeOptimizer::resolve_isconnected
    // (src/liboslexec/runtimeoptimize.cpp:2476-2505), before any folding: 1
    // when a connection feeds the parameter (or, with userdata_isconnected, it
    // is lockgeom=0), plus 2 when a later layer reads it or it is a renderer
    // output (ShadingSystemImpl::is_renderer_output, shadingsys.cpp:3832-3860)
    bool is_renderer_output(int li, const std::string& param) const {
        const std::string name2 = g.layers[(size_t)li].layername + "." + param;
        for (const SymLoc& sl : g.symlocs)
            if (sl.arena == ARENA_OUTPUTS && (sl.name == param || sl.name == name2)) return true;
        for (const std::string& ro : g.renderer_outputs)
            if (ro == param || ro == name2) return true;
        return false;
    }
    // A return inside a user function's body (between a functioncall op and
    // its end label, innermost call) returns from that function; elsewhere
    // it ends the layer (llvm_gen_return, batched_llvm_gen.cpp). Function
    // returns become "__fret" with imm[0] = the functioncall's index.
    bool mark_function_returns() {
        std::vector<std::pair<int, int>> open;  // (functioncall index, end)
        for (int k = 0; k < (int)lops.size(); ++k) {
            while (!open.empty() && k >= open.back().second) open.pop_back();
            LOp& op = lops[(size_t)k];
            if (op.name == "functioncall" || op.name == "functioncall_nr") {
                const int end = op.jumps.empty() ? k + 1 : op.jumps[0];
                if (end <= k || end > (int)lops.size()) return fail("functioncall with a bad end");
                open.push_back({ k, end });
            } else if (op.name == "return" && !open.empty()) {
                op.name = "__fret";
                op.imm[0] = open.back().first;
            }
        }
        return true;
    }

    void resolve_isconnected() {
        for (LOp& op : lops) {
            if (op.name != "isconnected" || op.args.size() < 2) continue;
            const GSym& s = syms[op.args[1]];
            int val = 0;
            if (s.layer >= 0 && (s.kind == SK_PARAM || s.kind == SK_OPARAM)) {
                const Layer& L = g.layers[(size_t)s.layer];
                bool up = false, down = false;
                for (const Connection& c : L.connections) up = up || c.dstparam == s.name;
                if (!up && ss.opts.userdata_isconnected) {
                    const int msi = L.master->find_symbol(s.name);
                    bool lockgeom = msi >= 0 ? L.master->symbols[(size_t)msi].lockgeom : true;
                    for (const InstanceParam& p : L.params)
                        if (p.name == s.name) lockgeom = p.lockgeom;
                    up = !lockgeom;
                }
                for (int lj = s.layer + 1; lj <= last_layer(); ++lj)
                    for (const Connection& c : g.layers[(size_t)lj].connections)
                        down = down || (c.srclayer == s.layer && c.srcparam == s.name);
                if (s.kind == SK_OPARAM && is_renderer_output(s.layer, s.name)) down = true;
                val = (up ? 1 : 0) + (down ? 2 : 0);
            }
            op.args = { op.args[0], const_int(val) };
            op.name = "assign";
            op.argrw = "wr";
        }
    }

    bool run(CompiledGroup& out) {
        if (g.layers.empty()) return fail("group has no layers");
        if (!build_lops()) return false;
        if (!mark_function_returns()) return false;
        resolve_isconnected();
        if (!prepare_messages()) return false;
        if (ss.opts.opt_constant_fold) fold_constants();
        if (ss.opts.opt_elide_useless_ops) eliminate_dead_ops();
        static_closures();
        analyze();
        assign_storage();
        if (!lower_all()) return false;
        // mask markers with nothing after them
        while (!ops.empty() && ops.back().code == OP_STORES_END) {
            ops.pop_back();
            op_names.pop_back();
        }
        // closure pools live after the symbol heap
        ProgramHeader h;
        std::memset(&h, 0, sizeof(h));
        h.magic = kProgramMagic;
        h.version = kProgramVersion;
        h.nops = (uint32_t)ops.size();
        h.nconst = (uint32_t)pool.size();
        h.closure_base = heap_top;
        h.max_comps = uses_closures ? (uint32_t)closure_nodes : 0u;
        h.max_terms = 0u;
        h.node_floats = wide_nodes ? (uint32_t)kNodeFloats : 0u;
        uint32_t closure_slots = uses_closures ? 1 + h.max_comps * node_floats(h) : 0;
        h.heap_slots = heap_top + closure_slots;
        if (h.heap_slots == 0) h.heap_slots = 1;
        h.flags = (uses_closures ? 1u : 0u);
        for (const GSym& s : syms)
            if (s.referenced && s.derivs) h.flags |= 2u;
        h.max_depth = max_depth;
        h.max_loop_iterations = (uint32_t)ss.opts.max_loop_iterations;
        out.retained_words = 0;
        for (const auto& r : g.retained)
            if (stop_layer < 0 || r->layer <= stop_layer) out.retained_words = std::max(out.retained_words, r->plane + r->words);
        h.flags |= program_tier() << 8;
        if (h.heap_slots > kArgOffsetMask) return fail("symbol heap too large");
        out.header = h;
        out.blob.resize(sizeof(h) + ops.size() * sizeof(Op) + pool.size() * 4);
        std::memcpy(out.blob.data(), &h, sizeof(h));
        if (!ops.empty()) std::memcpy(out.blob.data() + sizeof(h), ops.data(), ops.size() * sizeof(Op));
        if (!pool.empty())
            std::memcpy(out.blob.data() + sizeof(h) + ops.size() * sizeof(Op), pool.data(), pool.size() * 4);
        out.op_names = op_names;
        return true;
    }
};

}  // namespace

bool lower_group(ShadingSystem& ss, ShaderGroup& g, CompiledGroup& out, std::string& err, int stop_layer) {
    Lowerer L(ss, g, err);
    L.stop_layer = stop_layer;
    return L.run(out);
}

}  // namespace oslg
