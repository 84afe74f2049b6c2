#!/usr/bin/perl
# Test infrastructure: rewrites the PREPROCESSED reference translation unit on its way from
# `g++ -E` to the compiler (nothing is written to disk).  It
#  (1) turns CUDA launches `k<<<g, b>>>(args)` into lts_launch(k, g, b)(args) (host OpenMP);
#  (2) restores the Windows LLP64 reading of Geometry.cuh:17-23 (`*(long*)&y` reads 8 bytes
#      of a 4-byte float on LP64 Linux, corrupting the sign bit of the Quake-III rsqrt);
#  (3) adds recording calls around PathTracingIntegrator.cuh:41,55,107,
#      IntegratorHelper.cuh:69,107 and materials/textures/Procedural.cuh:166,186,295 so the driver can dump per-(pixel, sample) radiance and a
#      hash of the path's hit/visibility events and texture branch decisions (fBm/turbulence
#      octave count, marble colour segment) and the BSDF's grazing tests (reflect/transmit
#      against the geometric normal, BSDF.cuh:195,247; sameHemisphere, BxDF.cuh:126-128).  No arithmetic of the reference changes.
use strict; use warnings;
my %n = (launch => 0, llp64 => 0, begin => 0, hit => 0, vis => 0, mis => 0, sample => 0, octaves => 0, marble => 0, reflect => 0, hemi => 0);
while (my $l = <STDIN>) {
    $n{launch} += ($l =~ s/(\w+)\s*<<\s*<\s*(.*?)\s*>>\s*>\s*\(/lts_launch($1, $2)(/g);
    $n{llp64} += ($l =~ s/\*\s*\(\s*long\s*\*\s*\)\s*&\s*y\b/(long)*(int*)&y/g);
    $n{begin} += ($l =~ s/(Point2f filmSample = sampler->uniformSample\(id\);)/lts_hook_begin_sample(id, s); $1/);
    $n{hit} += ($l =~ s/(bool intersectionWithScene = scene->intersect\(r, &si\);)/$1 lts_hook_hit(intersectionWithScene ? (const void*)si.primitive : (const void*)0);/);
    $n{vis} += ($l =~ s/if \(!visibility\.unoccluded\(scene\)\)/if (!lts_hook_vis(visibility.unoccluded(scene)))/);
    $n{mis} += ($l =~ s/(bool foundSurfaceInteraction = scene\.intersect\(r, &lightIt\);)/$1 lts_hook_mis(foundSurfaceInteraction ? (const void*)lightIt.primitive : (const void*)0);/);
    $n{sample} += ($l =~ s/(d_camera->addSample\(pFilm, L\);)/lts_hook_sample(id, s, L.r, L.g, L.b); $1/);
    $n{octaves} += ($l =~ s/(int nInt = floorf\(n\);)/$1 lts_hook_branch(0x400000000ull + (unsigned)nInt);/);
    $n{reflect} += ($l =~ s/bool reflect = (dot\((?:wiW|\*wiWorld), ng\) \* dot\((?:woW|woWorld), ng\) > 0);/bool reflect = lts_hook_bool(0x600000000ull, $1);/g);
    $n{hemi} += ($l =~ s/return (w\.z \* wp\.z > 0);/return lts_hook_bool(0x700000000ull, $1);/);
    $n{marble} += ($l =~ s/(int first = \(int\)floorf\(t \* \(sizeof\(c\) \/ sizeof\(c\[0\]\) - 3\)\);)/$1 lts_hook_branch(0x500000000ull + (unsigned)first);/);
    print $l;
}
for my $k (sort keys %n) { die "instrument.pl: pattern '$k' not found in the reference\n" if $n{$k} < 1; }
print STDERR join(" ", map { "$_=$n{$_}" } sort keys %n), "\n";
