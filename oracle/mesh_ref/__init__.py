"""The reference's own .tfxmesh parser, compiled here (test infrastructure, a checker only).

TressFXBoneSkinning::LoadTressFXCollisionMeshData and the SuStringTokenizer it uses
(src/TressFX/TressFXBoneSkinning.cpp:36-285) parse a collision mesh.  The rest of that file needs the
engine interface, so build.py copies those two functions out of the reference tree at build time
(into the git-ignored oracle/_ref/) and compiles them unchanged in a minimal stand-in class; the
executable dumps what the parser loaded, in the layout of tests/cpp/mesh_dump.cpp (the library's own
loader), for tests/test_asset_pipeline.py to compare.
"""
from .build import EXE, available, build  # noqa: F401
