"""A simulation parameter file in FV3D's JSON layout with a Gmsh mesh, run
through the reference's program flow (set_solution, timedisc, output
files).  The file names are the caller's."""
from fv3d_gb300 import gmsh, params
sim = params.load_simulation("channel.json")
mesh = gmsh.read_msh("channel.msh")        # hexahedra, tetrahedra, prisms, pyramids; periodic links
u, stats, rows, files = params.run(sim, mesh, output_dir="out")
