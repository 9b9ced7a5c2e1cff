"""setmessage/getmessage between layers and getattribute against renderer
attributes, through the lowering and the oracle: found/not-found results,
destinations left unchanged, derivatives zeroed, the strict-message errors
of src/liboslexec/opmessage.cpp:19-138 (status bit, values unchanged),
the impossible-getmessage fold of src/liboslexec/constfold.cpp:2240-2258,
and getattribute folding (src/liboslexec/constfold.cpp:2262-2360)."""
import struct

import numpy as np
import pytest

from helpers import grid_globals, og, oracle_run, pixel_grid

ST_MESSAGE = 16


def opcodes(blob):
    import os
    import re
    src = open(os.path.join(os.path.dirname(__file__), "..", "openshadinglanguage_gb300", "csrc",
                            "oslg_program.h")).read()
    body = src.split("enum OpCode : uint16_t {")[1].split("};")[0]
    names = []
    for n in re.findall(r"\b(OP_[A-Z0-9_]+)\b", body):
        if n not in names:
            names.append(n)
    nops = struct.unpack("<I", blob[8:12])[0]
    return [names[struct.unpack("<H", blob[64 + 32 * i:66 + 32 * i])[0]] for i in range(nops)]


def sender(name="msg_send", double_set=False, guarded_m=False):
    """Layer 1: sets "col" (a color, only where u > 0.5) and "f" (u * 3,
    everywhere); optionally "f" a second time, and "m" under a condition
    that never holds."""
    b = og.OsoBuilder(name)
    k = b.param("float", "k", 0.7)
    kout = b.param("float", "kout", 0.0, output=True)
    b.op("assign", kout, k)
    u = b.glob("float", "u")
    half = b.const("float", 0.5)
    cond = b.tmp("int")
    b.op("gt", cond, u, half)
    c = b.tmp("color")
    one = b.const("float", 1.0)
    omu = b.tmp("float")
    b.op("sub", omu, one, u)
    b.op("color", c, u, k, omu)
    with b.if_(cond):
        b.op("setmessage", b.const("string", "col"), c)
    f = b.tmp("float")
    b.op("mul", f, u, b.const("float", 3.0))
    b.op("setmessage", b.const("string", "f"), f)
    if double_set:
        b.op("setmessage", b.const("string", "f"), one)
    if guarded_m:
        never = b.tmp("int")
        b.op("gt", never, u, b.const("float", 2.0))
        with b.if_(never):
            b.op("setmessage", b.const("string", "m"), one)
    return b.text()


def receiver(name="msg_recv", col_type="color", strict_probe=False):
    """Layer 2: Cout = message "col" (default 9), fv = message "f",
    found flags as ints; "never" was not set by anyone (folds to 0)."""
    b = og.OsoBuilder(name)
    kin = b.param("float", "kin", 0.0)
    kecho = b.param("float", "kecho", 0.0, output=True)
    b.op("assign", kecho, kin)  # the sender's output is used before any message is read
    cout = b.param(col_type, "Cout", 9.0, output=True)
    fv = b.param("float", "fv", -1.0, output=True)
    found = b.param("int", "found", -5, output=True)
    found2 = b.param("int", "found2", -5, output=True)
    found3 = b.param("int", "found3", -5, output=True)
    b.op("getmessage", found, b.const("string", "col"), cout)
    b.op("getmessage", found2, b.const("string", "f"), fv)
    x = b.tmp("float")
    b.op("getmessage", found3, b.const("string", "never"), x)
    if strict_probe:
        r1 = b.param("int", "r1", -5, output=True)
        r2 = b.param("int", "r2", -5, output=True)
        y = b.param("float", "y", -1.0, output=True)
        m = b.const("string", "m")
        b.op("getmessage", r1, m, x)  # "m" is possibly set (earlier, in a branch not taken)
        b.op("setmessage", m, b.const("float", 2.0))
        b.op("getmessage", r2, m, y)
    return b.text()


REC = [("Cout", og.TypeColor, 0, 12), ("fv", og.TypeFloat, 12, 4), ("found", og.TypeInt, 16, 4),
       ("found2", og.TypeInt, 20, 4), ("found3", og.TypeInt, 24, 4)]


def message_group(ss, tag, send_kw=None, recv_kw=None, extra=(), derivs=False, connect=True):
    """The sender layer feeds the receiver (kout -> kin): in the reference
    an upstream layer runs when its output is first used, and a layer with
    no outgoing connection is dropped."""
    ss.LoadMemoryCompiledShader("send_" + tag, sender("send_" + tag, **(send_kw or {})))
    ss.LoadMemoryCompiledShader("recv_" + tag, receiver("recv_" + tag, **(recv_kw or {})))
    g = ss.ShaderGroupBegin("g_" + tag)
    ss.Shader(g, "surface", "send_" + tag, "l1")
    ss.Shader(g, "surface", "recv_" + tag, "l2")
    if connect:
        ss.ConnectShaders(g, "l1", "kout", "l2", "kin")
    ss.ShaderGroupEnd(g)
    rec = list(REC) + list(extra)
    stride = 4 * 9 + 4 * (len(rec) - 1) if derivs else 4 + max(o for _, _, o, _ in rec)
    locs = []
    off = 0
    for nm, ty, o, sz in rec:
        d = derivs and nm == "Cout"
        locs.append(og.SymLocationDesc("l2." + nm, ty, d, og.SymArenaOutputs, off, stride))
        off += sz * (3 if d else 1)
    ss.add_symlocs(g, locs)
    return g, stride


def run(g, stride, W=16, H=8):
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, stride // 4), np.float32)
    st = oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out)
    return u, out, st


def test_messages_pass_between_layers():
    ss = og.ShadingSystem()
    g, stride = message_group(ss, "a")
    u, out, st = run(g, stride)
    assert st == 0
    ints = out.view(np.int32)
    set_ = u > 0.5
    col = np.stack([u, np.full_like(u, 0.7), (np.float32(1) - u).astype(np.float32)], 1)
    assert np.array_equal(out[set_, 0:3], col[set_])
    assert np.all(out[~set_, 0:3] == 9.0)  # not found: Cout keeps its value
    assert np.array_equal(ints[:, 4], set_.astype(np.int32))
    assert np.array_equal(out[:, 3], (u * np.float32(3)).astype(np.float32))
    assert np.all(ints[:, 5] == 1) and np.all(ints[:, 6] == 0)
    codes = opcodes(g.program_bytes())
    assert codes.count("OP_GETMESSAGE") == 2  # the "never" query folded to 0
    assert codes.count("OP_SETMESSAGE") == 2


def test_unconnected_layer_sends_no_messages():
    ss = og.ShadingSystem()
    g, stride = message_group(ss, "u", connect=False)
    u, out, st = run(g, stride)
    assert st == 0
    ints = out.view(np.int32)
    assert np.all(ints[:, 4] == 0) and np.all(ints[:, 5] == 0) and np.all(out[:, 0:3] == 9.0)
    assert "OP_SETMESSAGE" not in opcodes(g.program_bytes())


def test_found_message_zeroes_destination_derivatives():
    ss = og.ShadingSystem()
    g, stride = message_group(ss, "d", derivs=True)
    u, out, st = run(g, stride)
    assert st == 0
    set_ = u > 0.5
    assert np.all(out[set_, 3:9] == 0.0)
    assert np.all(out[~set_, 0:3] == 9.0) and np.all(out[~set_, 3:9] == 0.0)


def test_type_mismatch_is_an_error_and_not_found():
    ss = og.ShadingSystem()
    g, stride = message_group(ss, "t", recv_kw=dict(col_type="point"))
    u, out, st = run(g, stride)
    assert st & ST_MESSAGE
    assert np.all(out.view(np.int32)[:, 4] == 0) and np.all(out[:, 0:3] == 9.0)


def test_double_set_is_an_error_and_keeps_the_first_value():
    ss = og.ShadingSystem()
    g, stride = message_group(ss, "2", send_kw=dict(double_set=True))
    u, out, st = run(g, stride)
    assert st & ST_MESSAGE
    assert np.array_equal(out[:, 3], (u * np.float32(3)).astype(np.float32))


@pytest.mark.parametrize("strict", [1, 0])
def test_set_after_failed_query(strict):
    ss = og.ShadingSystem()
    ss.attribute("strict_messages", strict)
    extra = [("r1", og.TypeInt, 28, 4), ("r2", og.TypeInt, 32, 4), ("y", og.TypeFloat, 36, 4)]
    g, stride = message_group(ss, "s%d" % strict, send_kw=dict(guarded_m=True),
                              recv_kw=dict(strict_probe=True), extra=extra)
    u, out, st = run(g, stride)
    ints = out.view(np.int32)
    assert np.all(ints[:, 7] == 0)
    if strict:
        # queried before being set: the set is refused, later queries fail
        assert st & ST_MESSAGE
        assert np.all(ints[:, 8] == 0) and np.all(out[:, 9] == -1.0)
    else:
        assert st == 0
        assert np.all(ints[:, 8] == 1) and np.all(out[:, 9] == 2.0)


def test_message_name_must_be_constant():
    ss = og.ShadingSystem()
    b = og.OsoBuilder("varname")
    t = b.tmp("string")
    b.op("assign", t, b.const("string", "x"))
    u = b.glob("float", "u")
    cond = b.tmp("int")
    b.op("gt", cond, u, b.const("float", 0.5))
    with b.if_(cond):
        b.op("assign", t, b.const("string", "y"))
    o = b.param("float", "o", 0.0, output=True)
    b.op("setmessage", t, o)
    ss.LoadMemoryCompiledShader("varname", b.text())
    g = ss.ShaderGroupBegin("gv")
    ss.Shader(g, "surface", "varname", "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l1.o", og.TypeFloat, False, og.SymArenaOutputs, 0, 4)])
    with pytest.raises(og.OSLError, match="constant string"):
        g.program_bytes()


# ---- getattribute ---------------------------------------------------------------------------------

def attribute_shader(name="attrs"):
    b = og.OsoBuilder(name)
    outs = {}
    for nm, ty, d in [("fov", "float", -1.0), ("tint", "color", -1.0), ("id1", "int", -1),
                      ("missing", "float", 7.0), ("ver", "int", -1), ("layer_ok", "int", -1),
                      ("name_ok", "int", -1), ("wrongtype", "int", 3), ("group_ok", "int", -1)]:
        outs[nm] = b.param(ty, nm, d, output=True)
    res = {k: b.param("int", "r_" + k, -5, output=True) for k in ("fov", "tint", "id1", "missing", "ver",
                                                                   "wrongtype")}
    S = lambda s: b.const("string", s)
    b.op("getattribute", res["fov"], S("camera:fov"), outs["fov"])
    b.op("getattribute", res["tint"], S("obj1"), S("tint"), outs["tint"])
    b.op("getattribute", res["id1"], S("ids"), b.const("int", 1), outs["id1"])
    b.op("getattribute", res["missing"], S("nobody"), outs["missing"])
    b.op("getattribute", res["ver"], S("osl:version"), outs["ver"])
    b.op("getattribute", res["wrongtype"], S("camera:fov"), outs["wrongtype"])
    s1, s2, s3 = b.tmp("string"), b.tmp("string"), b.tmp("string")
    r = b.tmp("int")
    b.op("getattribute", r, S("shader:layername"), s1)
    b.op("eq", outs["layer_ok"], s1, S("l1"))
    b.op("getattribute", r, S("label"), s2)
    b.op("eq", outs["name_ok"], s2, S("hello"))
    b.op("getattribute", r, S("shader:groupname"), s3)
    b.op("eq", outs["group_ok"], s3, S("gattr"))
    return b.text()


ATTR_OUT = ["fov", "tint", "id1", "missing", "ver", "layer_ok", "name_ok", "wrongtype", "group_ok",
            "r_fov", "r_tint", "r_id1", "r_missing", "r_ver", "r_wrongtype"]


def attribute_group(ss, tag=""):
    ss.renderer_attribute("camera:fov", og.TypeFloat, 45.0)
    ss.renderer_attribute("tint", og.TypeColor, [0.1, 0.2, 0.3], object="obj1")
    ss.renderer_attribute("ids", og.TypeInt.array(3), [4, 5, 6])
    ss.renderer_attribute("label", og.TypeString, "hello")
    ss.LoadMemoryCompiledShader("attrs" + tag, attribute_shader("attrs" + tag))
    g = ss.ShaderGroupBegin("gattr")
    ss.Shader(g, "surface", "attrs" + tag, "l1")
    ss.ShaderGroupEnd(g)
    locs, off = [], 0
    types = {"tint": og.TypeColor, "fov": og.TypeFloat, "missing": og.TypeFloat}
    for nm in ATTR_OUT:
        ty = types.get(nm, og.TypeInt)
        locs.append(og.SymLocationDesc("l1." + nm, ty, False, og.SymArenaOutputs, off, 4 * 17))
        off += 12 if nm == "tint" else 4
    ss.add_symlocs(g, locs)
    return g


def check_attributes(out):
    ints = out.view(np.int32)
    assert np.all(out[:, 0] == 45.0)
    assert np.all(out[:, 1:4] == np.float32([0.1, 0.2, 0.3]))
    assert np.all(ints[:, 4] == 5)
    assert np.all(out[:, 5] == 7.0)
    assert np.all(ints[:, 6] == 11600)
    assert np.all(ints[:, 7] == 1) and np.all(ints[:, 8] == 1)
    assert np.all(ints[:, 9] == 3)  # float attribute read as int: not found, unchanged
    assert np.all(ints[:, 10] == 1)
    assert ints[:, 11:17].tolist() == [[1, 1, 1, 0, 1, 0]] * len(out)


def test_getattribute_folds_renderer_and_group_attributes():
    ss = og.ShadingSystem()
    g = attribute_group(ss)
    codes = opcodes(g.program_bytes())
    assert all(c in ("OP_ASSIGN", "OP_EQ", "OP_STORE_OUTPUT", "OP_LAYER_END", "OP_LOAD_GLOBAL") for c in codes)
    W, H = 8, 4
    u, v = pixel_grid(W, H, centers=True)
    out = np.zeros((W * H, 17), np.float32)
    assert oracle_run(g.program_bytes(), W * H, grid_globals(u, v, W, H, centers=True), out) == 0
    check_attributes(out)


def test_getattribute_needs_constant_names():
    ss = og.ShadingSystem()
    b = og.OsoBuilder("attrvar")
    nm = b.tmp("string")
    b.op("assign", nm, b.const("string", "a"))
    u = b.glob("float", "u")
    cond = b.tmp("int")
    b.op("gt", cond, u, b.const("float", 0.5))
    with b.if_(cond):
        b.op("assign", nm, b.const("string", "b"))
    o = b.param("float", "o", 0.0, output=True)
    r = b.param("int", "r", 0, output=True)
    b.op("getattribute", r, nm, o)
    ss.LoadMemoryCompiledShader("attrvar", b.text())
    g = ss.ShaderGroupBegin("gav")
    ss.Shader(g, "surface", "attrvar", "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("l1.r", og.TypeInt, False, og.SymArenaOutputs, 0, 4)])
    with pytest.raises(og.OSLError, match="must be constants"):
        g.program_bytes()


def userdata_attribute_group(ss, tag=""):
    """getattribute of per-point attributes the renderer passes in the
    userdata arena: a color with derivatives, an int, and the int read as
    a float (type mismatch: not found)."""
    b = og.OsoBuilder("uattr" + tag)
    c = b.param("color", "c", 0.0, output=True)
    i = b.param("int", "i", -1, output=True)
    f = b.param("float", "f", 5.0, output=True)
    r = [b.param("int", "r%d" % k, -5, output=True) for k in range(3)]
    S = lambda s: b.const("string", s)
    b.op("getattribute", r[0], S("uvw"), c)
    b.op("getattribute", r[1], S("objid"), i)
    b.op("getattribute", r[2], S("objid"), f)
    ss.LoadMemoryCompiledShader("uattr" + tag, b.text())
    g = ss.ShaderGroupBegin("guattr" + tag)
    ss.Shader(g, "surface", "uattr" + tag, "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("uvw", og.TypeColor, True, og.SymArenaUserData, 0, 40),
                       og.SymLocationDesc("objid", og.TypeInt, False, og.SymArenaUserData, 36, 40),
                       og.SymLocationDesc("l1.c", og.TypeColor, True, og.SymArenaOutputs, 0, 60),
                       og.SymLocationDesc("l1.i", og.TypeInt, False, og.SymArenaOutputs, 36, 60),
                       og.SymLocationDesc("l1.f", og.TypeFloat, False, og.SymArenaOutputs, 40, 60)]
                  + [og.SymLocationDesc("l1.r%d" % k, og.TypeInt, False, og.SymArenaOutputs, 44 + 4 * k, 60)
                     for k in range(3)])
    return g


def userdata_records(n, seed=21):
    rng = np.random.default_rng(seed)
    ud = rng.normal(size=(n, 10)).astype(np.float32)
    ud.view(np.int32)[:, 9] = rng.integers(0, 1000, n)
    return ud


def check_userdata_attributes(out, ud):
    assert np.array_equal(out[:, 0:9].view(np.uint32), ud[:, 0:9].view(np.uint32))
    ints = out.view(np.int32)
    assert np.array_equal(ints[:, 9], ud.view(np.int32)[:, 9])
    assert np.all(out[:, 10] == 5.0)
    assert ints[:, 11:14].tolist() == [[1, 1, 0]] * len(out)


def test_getattribute_reads_per_point_userdata():
    ss = og.ShadingSystem()
    g = userdata_attribute_group(ss)
    n = 200
    ud = userdata_records(n)
    out = np.zeros((n, 15), np.float32)
    assert oracle_run(g.program_bytes(), n, og.make_globals(u=0.5), out, userdata=ud) == 0
    check_userdata_attributes(out, ud)


@pytest.mark.parametrize("with_derivs", [False, True])
def test_userdata_parameter_derivatives(with_derivs):
    """A varying parameter read from userdata whose derivatives are needed
    downstream (Dx): the record's derivatives when it carries them, else 0
    (never the words that follow the value)."""
    ss = og.ShadingSystem()
    b = og.OsoBuilder("udd%d" % with_derivs)
    q = b.param("float", "q", 0.0, lockgeom=False)
    o = b.param("float", "o", 0.0, output=True)
    d = b.param("float", "d", 0.0, output=True)
    b.op("assign", o, q)
    b.op("Dx", d, q)
    ss.LoadMemoryCompiledShader("udd%d" % with_derivs, b.text())
    g = ss.ShaderGroupBegin("gudd%d" % with_derivs)
    ss.Shader(g, "surface", "udd%d" % with_derivs, "l1")
    ss.ShaderGroupEnd(g)
    ss.add_symlocs(g, [og.SymLocationDesc("q", og.TypeFloat, with_derivs, og.SymArenaUserData, 0, 12),
                       og.SymLocationDesc("l1.o", og.TypeFloat, False, og.SymArenaOutputs, 0, 8),
                       og.SymLocationDesc("l1.d", og.TypeFloat, False, og.SymArenaOutputs, 4, 8)])
    n = 64
    ud = np.random.default_rng(1).normal(size=(n, 3)).astype(np.float32)
    out = np.zeros((n, 2), np.float32)
    assert oracle_run(g.program_bytes(), n, og.make_globals(u=0.5), out, userdata=ud) == 0
    assert np.array_equal(out[:, 0], ud[:, 0])
    assert np.array_equal(out[:, 1], ud[:, 1] if with_derivs else np.zeros(n, np.float32))


def message_testsuite_group(ss):
    """testsuite/message-no-closure's a.osl -> b.osl as a group; returns
    (group, floats per output record)."""
    a = og.OsoBuilder("msg_a")
    S = lambda b, s: b.const("string", s)
    kd = a.param("float", "Kd", 0.5)
    f_out = a.param("float", "f_out", 0.0, output=True)
    c_out = a.param("color", "c_out", 0.0, output=True)
    a.op("assign", f_out, kd)
    h = a.tmp("float")
    a.op("div", h, kd, a.const("float", 2.0))
    a.op("color", c_out, h, a.const("float", 1.0), a.const("float", 1.0))
    half = a.tmp("color")
    a.op("div", half, c_out, a.const("float", 2.0))
    a.op("setmessage", S(a, "foo"), half)
    arr = a.param("float[4]", "arr", [42.0, 43.0, 44.0, 45.0])
    a.op("setmessage", S(a, "array"), arr)
    wd = a.param("int", "wd", -7, output=True)
    wc = a.tmp("int")
    a.op("getmessage", wd, S(a, "wrong_direction_test"), wc)
    b = og.OsoBuilder("msg_b")
    f_in = b.param("float", "f_in", 41.0)
    c_in = b.param("color", "c_in", 42.0)
    outs = {nm: b.param(ty, nm, 0.0 if ty != "int" else -7, output=True)
            for nm, ty in [("foo", "color"), ("r_foo", "int"), ("bar", "float"), ("r_bar", "int"),
                           ("r_wrong", "int"), ("array", "float[4]"), ("r_array", "int"), ("Cout", "color"),
                           ("fin", "float")]}
    b.op("assign", outs["fin"], f_in)
    b.op("assign", outs["foo"], b.const("float", 0.0))
    b.op("setmessage", S(b, "wrong_direction_test"), b.const("int", 3))
    b.op("getmessage", outs["r_foo"], S(b, "foo"), outs["foo"])
    b.op("getmessage", outs["r_bar"], S(b, "bar"), outs["bar"])
    b.op("getmessage", outs["r_wrong"], S(b, "foo"), outs["bar"])
    b.op("getmessage", outs["r_array"], S(b, "array"), outs["array"])
    c = b.local("int", "c")
    b.op("assign", c, b.const("int", 0))
    b.op("getmessage", b.tmp("int"), S(b, "already_queried"), c)
    b.op("setmessage", S(b, "already_queried"), b.const("int", 3))
    b.op("setmessage", S(b, "message_on_same_layer"), b.const("int", 3))
    b.op("getmessage", b.tmp("int"), S(b, "message_on_same_layer"), c)
    b.op("setmessage", S(b, "set_twice"), b.const("int", 3))
    b.op("setmessage", S(b, "set_twice"), b.const("int", 4))
    N = b.glob("normal", "N")
    b.op("setmessage", S(b, "set_get_int"), N)
    b.op("getmessage", b.tmp("int"), S(b, "set_get_int"), c)
    diff = b.local("color", "diff")
    b.op("assign", diff, b.const("float", 0.0))
    b.op("setmessage", S(b, "get_int_set"), b.const("int", 3))
    b.op("getmessage", b.tmp("int"), S(b, "get_int_set"), diff)
    fc, nc = b.tmp("float"), b.tmp("color")
    b.op("assign", fc, c)
    b.op("mul", nc, N, fc)
    b.op("add", outs["Cout"], nc, diff)
    ss.LoadMemoryCompiledShader("msg_a", a.text())
    ss.LoadMemoryCompiledShader("msg_b", b.text())
    g = ss.ShaderGroupBegin("gmsg")
    ss.Shader(g, "surface", "msg_a", "alayer")
    ss.Shader(g, "surface", "msg_b", "blayer")
    ss.ConnectShaders(g, "alayer", "f_out", "blayer", "f_in")
    ss.ConnectShaders(g, "alayer", "c_out", "blayer", "c_in")
    ss.ShaderGroupEnd(g)
    layout = [("blayer.foo", og.TypeColor, 3), ("blayer.r_foo", og.TypeInt, 1), ("blayer.bar", og.TypeFloat, 1),
              ("blayer.r_bar", og.TypeInt, 1), ("blayer.r_wrong", og.TypeInt, 1),
              ("blayer.array", og.TypeFloat.array(4), 4), ("blayer.r_array", og.TypeInt, 1),
              ("blayer.Cout", og.TypeColor, 3), ("blayer.fin", og.TypeFloat, 1), ("alayer.wd", og.TypeInt, 1)]
    locs, off = [], 0
    for nm, ty, nw in layout:
        locs.append(og.SymLocationDesc(nm, ty, False, og.SymArenaOutputs, off, 4 * 17))
        off += 4 * nw
    ss.add_symlocs(g, locs)
    return g, 17


def test_message_no_closure_testsuite_case():
    """testsuite/message-no-closure (a.osl -> b.osl, optimized: ref
    out-opt.txt): the color message 'foo' = c_out / 2 = (0.125, 0.5, 0.5)
    arrives; 'bar' was never sent (0, destination unchanged); 'foo' read as
    a float is a type mismatch (0, unchanged); the float[4] message arrives
    whole; a query before any send is folded away, so setting the message
    afterwards is no error; a message set and read in the same layer
    arrives; setting twice and reading as another type are errors."""
    ss = og.ShadingSystem()
    g, rec = message_testsuite_group(ss)
    n = 16
    Nv = np.random.default_rng(2).normal(size=(3, n)).astype(np.float32)
    out = np.zeros((n, 17), np.float32)
    st = oracle_run(g.program_bytes(), n, og.make_globals(N=Nv, u=0.25, v=0.75), out)
    ints = out.view(np.int32)
    assert st & ST_MESSAGE  # set_twice and the two type mismatches
    assert np.all(out[:, 0:3] == np.float32([0.125, 0.5, 0.5])) and np.all(ints[:, 3] == 1)
    assert np.all(out[:, 4] == 0.0) and np.all(ints[:, 5] == 0) and np.all(ints[:, 6] == 0)
    assert np.all(out[:, 7:11] == np.float32([42, 43, 44, 45])) and np.all(ints[:, 11] == 1)
    assert np.array_equal(out[:, 12:15], (Nv.T * np.float32(3.0)).astype(np.float32))
    assert np.all(out[:, 15] == 0.5)
    assert np.all(ints[:, 16] == 0)
