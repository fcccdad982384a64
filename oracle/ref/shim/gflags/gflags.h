// Empty stand-in for gflags: the reference headers include it but define no flags.
#pragma once
