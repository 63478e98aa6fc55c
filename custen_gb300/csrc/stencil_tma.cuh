// TMA staging path of the stencil kernel (filled in once the plain-load path is parity-checked).
#pragma once
