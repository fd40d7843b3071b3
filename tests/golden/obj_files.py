"""A small OBJ/MTL pair written for the loader tests (this project's own content, not a
file of the reference): two objects, a material file with Windows line endings, faces in
the three vertex forms (v, v//vn, v/vt/vn), a quad, an unknown `usemtl` name, a face
before the second object's first `usemtl`, the px/py keys, comments and blank lines."""
import os

MTL = ("# materials\r\n"
       "newmtl white\r\n"
       "kd 0.8 0.8 0.8\r\n"
       "\r\n"
       "newmtl glass\r\n"
       "ke 0 0 0\r\n"
       "kd 0 0 0\r\n"
       "ks 0.04 0.04 0.04\r\n"
       "n 1.5\r\n"
       "px 7\r\n"
       "py 3\r\n"
       "alpha_x 0.25\r\n"
       "is_specular 1\r\n"
       "is_transmissive 1\r\n")

OBJ = """# loader test scene
mtllib test_scene.mtl

o Walls
v -1 -1 -1
v 1 -1 -1
v 1 1 -1
v -1 1 -1
v -1 -1 1
v 1 -1 1
vt 0 0
vt 1 0
vt 1 1
vt 0 1
vn 0 0 1
vn 0 1 0
usemtl white
f 1//1 2//1 3//1
f 1//1 3//1 4//1
usemtl no-such-material
f 1/1/2 2/2/2 6/3/2 5/4/2

o Box
f 5 6 2
usemtl glass
f 4//1 3//1 2//1
"""


# triangles (in file order) whose face gives no normal indices: the reference leaves their
# normals unset, this loader writes zeros
NO_NORMALS = (3,)


def write(directory):
    """Writes test_scene.obj and test_scene.mtl into `directory`; returns the OBJ path."""
    with open(os.path.join(directory, "test_scene.mtl"), "wb") as f:
        f.write(MTL.encode())
    path = os.path.join(directory, "test_scene.obj")
    with open(path, "w") as f:
        f.write(OBJ)
    return path
