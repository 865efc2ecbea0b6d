// Empty stand-in for <gmsh.h> (reference-pin builds only): the reference
// headers that include it declare the gmsh-based mesh generator but use no
// gmsh type in the code the pins compile.
#pragma once
