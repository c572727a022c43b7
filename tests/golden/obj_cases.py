"""OBJ texts and readobj options shared by make_golden_obj.py (which runs the
reference's reader) and tests/test_obj.py (which runs this package's)."""

CUBE = b"""# cube with quads, uvs and normals
mtllib cube.mtl
v -1 -1 -1
v 1 -1 -1
v 1 1 -1
v -1 1 -1
v -1 -1 1
v 1 -1 1
v 1 1 1
v -1 1 1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 -1
vn 0 0 1
vn 0 -1 0
vn 1 0 0
vn 0 1 0
vn -1 0 0
usemtl red
f 1/1/1 4/4/1 3/3/1 2/2/1
f 5/1/2 6/2/2 7/3/2 8/4/2
usemtl blue
f 1/1/3 2/2/3 6/3/3 5/4/3
f 2/1/4 3/2/4 7/3/4 6/4/4
s off
f 3/1/5 4/2/5 8/3/5 7/4/5
f 4/1/6 1/2/6 5/3/6 8/4/6
"""

POLY = b"""o poly
v 0 0 0
v 1 0 0
v 1.5 0.8 0.1
v 0.7 1.4 0.2
v -0.3 0.9 0.1
v 2 2 2
vn 0 0 1
f 1//1 2//1 3//1 4//1 5//1
f 2//1 6//1 3//1
vt 0.5 0.5 0.0
f 1/1/1 2/1/1 6/1/1
"""

PLAIN = b"""v 0 0 0
v 1 0 0
v 0 1 0
v 1 1 0.5
f 1 2 3
f 2 4 3
"""

NOTHING = b"""# no geometry
g empty
"""

CASES = [
    ('cube', CUBE, dict()),
    ('cube_orient', CUBE, dict(orient='-xZy')),
    ('cube_scale', CUBE, dict(scale=0.5)),
    ('poly', POLY, dict()),
    ('poly_auto', POLY, dict(scale='auto', orient='Yzx')),
    ('poly_quadless', POLY, dict(usemtl=False)),
    ('plain', PLAIN, dict(simple=False)),
    ('nothing', NOTHING, dict()),
]
