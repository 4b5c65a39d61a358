"""save() of generated programs in its three formats (abl_save in
openabl_gb300/csrc/abl_host.cpp), checked on the CPU against the layouts the
reference runtime writes (asset/c/libabl.c:46-231):

* SAVE_JSON: {"Type":[{"m":v,...},\\n{...}],...} with %f floats and
  true/false booleans (libabl.c:46-124);
* SAVE_FLAME_XML: <states>\\n<itno>0</itno>\\n, then per agent an <xagent>
  with <name>, one element per member, vectors split into <m_x>/<m_y>/<m_z>,
  booleans as integers (libabl.c:126-209);
* SAVE_FLAMEGPU_XML: the same, except that the position member is written
  as <x>, <y>, <z> (z 0.0 in 2D).

The expected text is built here, independently, from those rules; records
are laid out as the generated programs lay them out (C structs).
"""
import ctypes

import pytest

import openabl_gb300 as o

T_END, T_BOOL, T_INT, T_FLOAT, T_STRING, T_FLOAT2, T_FLOAT3 = range(7)


class TypeInfo(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int), ("offset", ctypes.c_uint), ("name", ctypes.c_char_p),
                ("is_pos", ctypes.c_bool)]


class AgentInfo(ctypes.Structure):
    _fields_ = [("info", ctypes.POINTER(TypeInfo)), ("offset", ctypes.c_uint),
                ("name", ctypes.c_char_p)]


class DynArray(ctypes.Structure):
    _fields_ = [("values", ctypes.c_void_p), ("len", ctypes.c_size_t), ("cap", ctypes.c_size_t)]


class Cell(ctypes.Structure):   # {float2 pos; bool alive; int kind; float energy}
    _fields_ = [("pos", ctypes.c_double * 2), ("alive", ctypes.c_bool), ("kind", ctypes.c_int),
                ("energy", ctypes.c_double)]


class Bird(ctypes.Structure):   # {float3 pos; float3 velocity}
    _fields_ = [("pos", ctypes.c_double * 3), ("velocity", ctypes.c_double * 3)]


class Agents(ctypes.Structure):
    _fields_ = [("cells", DynArray), ("birds", DynArray)]


CELL_INFO = [(T_FLOAT2, Cell.pos.offset, b"pos", True), (T_BOOL, Cell.alive.offset, b"alive", False),
             (T_INT, Cell.kind.offset, b"kind", False),
             (T_FLOAT, Cell.energy.offset, b"energy", False)]
BIRD_INFO = [(T_FLOAT3, Bird.pos.offset, b"pos", True),
             (T_FLOAT3, Bird.velocity.offset, b"velocity", False)]


def _type_table(members, size):
    arr = (TypeInfo * (len(members) + 1))()
    for k, (t, off, name, is_pos) in enumerate(members):
        arr[k] = TypeInfo(t, off, name, is_pos)
    arr[len(members)] = TypeInfo(T_END, size, None, False)  # END carries the record size
    return arr


def population():
    cells = (Cell * 3)(Cell((1.5, 2.25), True, 3, 0.125), Cell((0.0, -7.0), False, -2, 1e-7),
                       Cell((123.456789, 9.0), True, 0, -3.5))
    birds = (Bird * 2)(Bird((1.0, 2.0, 3.0), (-0.5, 0.25, 0.0)),
                       Bird((4.5, 5.5, 6.5), (1e3, -1e-3, 2.0)))
    agents = Agents(DynArray(ctypes.cast(cells, ctypes.c_void_p), 3, 3),
                    DynArray(ctypes.cast(birds, ctypes.c_void_p), 2, 2))
    cinfo = _type_table(CELL_INFO, ctypes.sizeof(Cell))
    binfo = _type_table(BIRD_INFO, ctypes.sizeof(Bird))
    ainfo = (AgentInfo * 3)(AgentInfo(cinfo, Agents.cells.offset, b"Cell"),
                            AgentInfo(binfo, Agents.birds.offset, b"Bird"),
                            AgentInfo(None, 0, None))
    keep = (cells, birds, cinfo, binfo)
    return agents, ainfo, keep, [("Cell", cells, CELL_INFO), ("Bird", birds, BIRD_INFO)]


def expected_json(types):
    out = []
    for name, recs, members in types:
        items = []
        for r in recs:
            fields = []
            for t, _, m, _ in members:
                v = getattr(r, m.decode())
                if t == T_BOOL:
                    s = "true" if v else "false"
                elif t == T_INT:
                    s = "%d" % v
                elif t == T_FLOAT:
                    s = "%f" % v
                else:
                    s = "[" + ",".join("%f" % x for x in v) + "]"
                fields.append('"%s":%s' % (m.decode(), s))
            items.append("{" + ",".join(fields) + "}")
        out.append('"%s":[' % name + ",\n".join(items) + "]")
    return "{" + ",".join(out) + "}"


def expected_xml(types, for_gpu):
    s = "<states>\n<itno>0</itno>\n"
    for name, recs, members in types:
        for r in recs:
            s += "<xagent>\n<name>%s</name>\n" % name
            for t, _, m, is_pos in members:
                nm, v = m.decode(), getattr(r, m.decode())
                if for_gpu and is_pos:
                    s += "<x>%f</x>\n<y>%f</y>\n" % (v[0], v[1])
                    s += ("<z>%f</z>\n" % v[2]) if t == T_FLOAT3 else "<z>0.0</z>\n"
                elif t in (T_BOOL, T_INT):
                    s += "<%s>%d</%s>\n" % (nm, int(v), nm)
                elif t == T_FLOAT:
                    s += "<%s>%f</%s>\n" % (nm, v, nm)
                else:
                    for ax, x in zip("xyz", v):
                        s += "<%s_%s>%f</%s_%s>\n" % (nm, ax, x, nm, ax)
            s += "</xagent>\n"
    return s + "</states>\n"


@pytest.fixture(scope="module")
def abl_save():
    f = o.library().abl_save
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_int]
    return f


@pytest.mark.parametrize("fmt", [0, 1, 2])
def test_save_writes_the_reference_layout(abl_save, tmp_path, fmt):
    agents, ainfo, keep, types = population()
    path = tmp_path / "out.txt"
    assert abl_save(ctypes.addressof(agents), ctypes.addressof(ainfo), str(path).encode(), fmt,
                    8) == 0
    want = expected_json(types) if fmt == 0 else expected_xml(types, for_gpu=fmt == 2)
    assert path.read_text() == want


def test_save_refuses_unknown_formats_and_paths(abl_save, tmp_path):
    agents, ainfo, keep, _ = population()
    assert abl_save(ctypes.addressof(agents), ctypes.addressof(ainfo),
                    str(tmp_path / "x").encode(), 7, 8) == -1
    assert not (tmp_path / "x").exists()
    assert abl_save(ctypes.addressof(agents), ctypes.addressof(ainfo),
                    str(tmp_path / "no" / "such" / "dir").encode(), 0, 8) == -1
