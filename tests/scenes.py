"""Small seeded scenes shared by the tests (built through the product's host C ABI)."""
import lavaframe_gb300 as lf

GENERATED = {
    "soup": lambda s: s.gen_soup(4096, 10, 1),
    "icospheres": lambda s: s.gen_icospheres(5, 4, 3, 64, 32),
    "cornell": lambda s: s.gen_cornell(64, 64),
    "room": lambda s: s.gen_room(2000, 4),
}


def build(name, **kw):
    s = lf.HostScene()
    GENERATED[name](s) if not kw else kw["fn"](s)
    s.build()
    return s
