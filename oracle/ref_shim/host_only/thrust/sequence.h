// Empty stand-in (reference-pin builds only): the reference header that
// includes it declares plain device pointers and uses nothing from thrust.
#pragma once
